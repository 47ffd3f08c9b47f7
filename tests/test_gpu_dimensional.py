"""GPU parity of the dimensional (v18) kernels and time step against the oracle.

The material laws' exponentials (10^x of the viscosity, e^x of the
permeability) are the library's own (expo.h), compiled into the device code
and into the oracle alike, so every kernel is compared bit for bit and a full
time step to 1e-12 (relative, max-norm) with identical iteration counts."""
import ctypes

import numpy as np
import pytest

import hydrothermal3d_gb300 as ht
from hydrothermal3d_gb300 import api, abi, v18
from conftest import rel_err, no_edges_mask

pytestmark = pytest.mark.gpu


def same(got, ref):
    np.testing.assert_array_equal(got, ref)


def setup(n=(9, 8, 7), seed=3):
    b = v18.box(*n, seed=seed, nitout=50, tol=1e-9)
    rng = np.random.default_rng(seed)
    # phases: mostly crust, a fault (2), a pluton (3), air on top, an immersed layer (-1)
    nx, ny, nz = n
    phc = b["phc"].copy(order="F")
    phc[3:5, 2:4, 2:4] = 2.0
    phc[5:7, 3:5, 3:5] = 3.0
    phc[:, -2, :] = -1.0
    phv = np.asfortranarray(np.where(rng.uniform(size=(nx + 1, ny + 1, nz + 1)) < 0.2, 2.0, 0.0))
    phv[:, -1, :] = 1.0
    b["phc2"], b["phv2"] = phc, phv
    b["wN2"] = np.asfortranarray(rng.uniform(0.3, 0.9, (nx + 2, nz + 2)))
    return b


def test_material_laws(ctx, orc):
    rng = np.random.default_rng(1)
    a = np.asfortranarray(rng.uniform(300, 900, (50, 1, 1)))
    b = np.asfortranarray(rng.uniform(1e5, 3e8, (50, 1, 1)))
    for which in range(12):
        aa = a - 273.15 if which in (5, 6) else (np.asfortranarray(rng.uniform(-5, 0, a.shape)) if which == 8 else a)
        bb = b if which in (5, 6) else (np.full(a.shape, 3.0, order="F") if which == 8 else b)
        if which == 9:
            aa = np.asfortranarray(rng.integers(-1, 4, a.shape).astype(float))
            bb = np.full(a.shape, 0.01, order="F")
        if which == 10:
            aa = np.asfortranarray(rng.uniform(-740, 705, a.shape))
        if which == 11:
            aa = np.asfortranarray(rng.uniform(-320, 305, a.shape))
        got = ht.to_numpy(api.material_law(ctx, which, ht.from_numpy(aa), ht.from_numpy(bb)))
        ref = np.array([orc.law(which, x, y) for x, y in zip(aa.ravel(), bb.ravel())]).reshape(aa.shape)
        same(got, ref)


def test_exponentials_within_cuda_error_bounds(ctx):
    """The library's e^x and 10^x against CUDA's exp and pow(10, x) (documented
    at 1 and 2 ulp of the exact value): within 2 ulp of CUDA's, and equal to
    CUDA's exp for most arguments (both are then correctly rounded)."""
    import torch
    rng = np.random.default_rng(2)
    for which, lo, hi, fn in ((10, -700.0, 700.0, torch.exp), (11, -300.0, 300.0, lambda t: torch.pow(10.0, t))):
        x = np.asfortranarray(rng.uniform(lo, hi, (4096, 1, 1)))
        got = ht.to_numpy(api.material_law(ctx, which, ht.from_numpy(x)))
        cuda = fn(ht.from_numpy(x)).cpu().numpy()
        ulps = np.abs(got - cuda) / np.spacing(np.abs(cuda))
        assert ulps.max() <= 2.0, (which, ulps.max())
        if which == 10:
            assert (ulps == 0).mean() > 0.9


def test_property_kernels(ctx, orc):
    b = setup()
    p = b["params"]
    nx, ny, nz = (s - 2 for s in b["T"].shape)
    T, P, phc, phv = b["T"], b["P"], b["phc2"], b["phv2"]
    Td, Pd, phcd, phvd = ht.from_numpy(T), ht.from_numpy(P), ht.from_numpy(phc), ht.from_numpy(phv)
    kv, kvd = np.zeros((nx + 1, ny + 1, nz + 1), order="F"), ht.zeros(nx + 1, ny + 1, nz + 1)
    orc.call("ComputeThermalConductivity", kv, T, phv, p.phi_i, p.sc_kt, p.sc_T, nx, ny, nz)
    api.ComputeThermalConductivity(ctx, kvd, Td, phvd, p.phi_i, p.sc_kt, p.sc_T)
    same(ht.to_numpy(kvd), kv)
    import ctypes
    for mode in (1, 2, 3):
        for kmul in (None, b["kmul"]):
            orc.call("ComputeHydroConductivity", kv, T, P, phv, p.ymin, p.dy, p.k_fact, 3000.0 / p.sc_L, p.sc_sigma,
                     p.sc_T, p.sc_L, p.sc_t, p.sc_eta, ctypes.c_int(mode), kmul, nx, ny, nz)
            api.ComputeHydroConductivity(ctx, kvd, Td, Pd, phvd, p.ymin, p.dy, p.k_fact, 3000.0 / p.sc_L, p.sc_sigma,
                                         p.sc_T, p.sc_L, p.sc_t, p.sc_eta, mode,
                                         None if kmul is None else ht.from_numpy(kmul))
            same(ht.to_numpy(kvd), kv)
    orc.call("ComputeFluidDensity", kv, T, P, phv, p.sc_sigma, p.sc_T, p.sc_rho, nx, ny, nz)
    api.ComputeFluidDensity(ctx, kvd, Td, Pd, phvd, p.sc_sigma, p.sc_T, p.sc_rho)
    same(ht.to_numpy(kvd), kv)
    c, cd = np.zeros((nx, ny, nz), order="F"), ht.zeros(nx, ny, nz)
    orc.call("SmoothConductivityV2C", c, kv, nx, ny, nz)
    api.SmoothConductivityV2C(ctx, cd, kvd)
    same(ht.to_numpy(cd), c)
    orc.call("SmoothConductivityC2V", kv, c, nx, ny, nz)
    api.SmoothConductivityC2V(ctx, kvd, cd)
    same(ht.to_numpy(kvd), kv)
    k = [np.zeros(s, order="F") for s in ((nx + 1, ny, nz), (nx, ny + 1, nz), (nx, ny, nz + 1))]
    kd = [ht.zeros(*a.shape) for a in k]
    orc.call("InitConductivity", *k, kv, nx, ny, nz)
    api.InitConductivity(ctx, *kd, kvd)
    for a, bb in zip(kd, k):
        same(ht.to_numpy(a), bb)
    rC, rCd = np.zeros((nx, ny, nz), order="F"), ht.zeros(nx, ny, nz)
    orc.call("ComputeRhoCeffective", rC, T, P, phc, p.phi_i, p.sc_T, p.sc_sigma, p.sc_C, p.sc_rho, nx, ny, nz)
    api.ComputeRhoCeffective(ctx, rCd, Td, Pd, phcd, p.phi_i, p.sc_T, p.sc_sigma, p.sc_C, p.sc_rho)
    same(ht.to_numpy(rCd), rC)
    Tc0 = np.asfortranarray(T[1:-1, 1:-1, 1:-1] * 0.995)
    Pc0 = np.asfortranarray(P[1:-1, 1:-1, 1:-1] * 1.003)
    o, od = np.zeros((nx, ny, nz), order="F"), ht.zeros(nx, ny, nz)
    orc.call("phi_rhof", o, Tc0, Pc0, phc, p.phi_i, p.sc_rho, p.sc_T, p.sc_sigma, ctypes.c_int(1), ctypes.c_int(0),
             nx, ny, nz)
    api.PhiRhofOld(ctx, od, ht.from_numpy(Tc0), ht.from_numpy(Pc0), phcd, p.phi_i, p.sc_rho, p.sc_T, p.sc_sigma)
    same(ht.to_numpy(od), o)
    for name, args, cell in (("PhiRhof", (T, P), 0), ("PhiDrhodP", (T, P), 0)):
        o, od = np.zeros((nx, ny, nz), order="F"), ht.zeros(nx, ny, nz)
        orc.call("phi_rhof", o, *args, phc, p.phi_i, p.sc_rho, p.sc_T, p.sc_sigma, ctypes.c_int(cell),
                 ctypes.c_int(1 if name == "PhiDrhodP" else 0), nx, ny, nz)
        getattr(api, name)(ctx, od, Td, Pd, phcd, p.phi_i, p.sc_rho, p.sc_T, p.sc_sigma)
        same(ht.to_numpy(od), o)


def test_boundary_kernels_snapshot_semantics(ctx, orc):
    b = setup()
    p = b["params"]
    nx, ny, nz = (s - 2 for s in b["T"].shape)
    rng = np.random.default_rng(9)
    ky = np.asfortranarray(rng.uniform(0.5, 2, (nx, ny + 1, nz)))
    T = b["T"] + np.asfortranarray(rng.uniform(-0.01, 0.01, b["T"].shape))
    To, Td = T.copy(order="F"), ht.from_numpy(T)
    orc.call("SetTemperatureBCs_dim", To, ky, b["wN2"], b["phc2"], p.qyS, 1 / p.dy, p.Ttop, nx, ny, nz)
    api.SetTemperatureBCs(ctx, Td, ht.from_numpy(ky), ht.from_numpy(b["wN2"]), ht.from_numpy(b["phc2"]), p.qyS,
                          1 / p.dy, 1.0, p.Tbot, p.Ttop)
    np.testing.assert_array_equal(ht.to_numpy(Td), To)
    P = b["P"] * (1 + np.asfortranarray(rng.uniform(-0.01, 0.01, b["P"].shape)))
    Po, Pd = P.copy(order="F"), ht.from_numpy(P)
    orc.call("SetPressureBCs_dim", Po, b["wN2"], b["phc2"], p.Ptop, nx, ny, nz)
    api.SetPressureBCs_dim(ctx, Pd, ht.from_numpy(b["wN2"]), ht.from_numpy(b["phc2"]), p.Pbot, p.Ptop)
    np.testing.assert_array_equal(ht.to_numpy(Pd), Po)


def test_boundary_kernels_read_cells_they_overwrite(ctx, orc):
    """Rules that read a cell the same call overwrites (an air cell next to a
    face ghost, an immersed cell above another immersed or air cell) must see
    its value from before the call, as the oracle's explicit snapshot does."""
    b = setup()
    p = b["params"]
    nx, ny, nz = (s - 2 for s in b["T"].shape)
    phc = b["phc2"].copy(order="F")
    phc[1, 3, 2] = phc[nx, 2, 3] = phc[2, 1, 3] = phc[3, 4, 1] = phc[4, 2, nz] = 1.0  # air read by x/y/z face rules
    phc[4, 5, 4] = phc[4, 6, 4] = -1.0  # immersed above immersed
    phc[5, 3, 5], phc[5, 4, 5] = 1.0, -1.0  # immersed above air
    rng = np.random.default_rng(19)
    ky = np.asfortranarray(rng.uniform(0.5, 2, (nx, ny + 1, nz)))
    T = b["T"] + np.asfortranarray(rng.uniform(-0.01, 0.01, b["T"].shape))
    To, Td = T.copy(order="F"), ht.from_numpy(T)
    orc.call("SetTemperatureBCs_dim", To, ky, b["wN2"], phc, p.qyS, 1 / p.dy, p.Ttop, nx, ny, nz)
    api.SetTemperatureBCs(ctx, Td, ht.from_numpy(ky), ht.from_numpy(b["wN2"]), ht.from_numpy(phc), p.qyS,
                          1 / p.dy, 1.0, p.Tbot, p.Ttop)
    np.testing.assert_array_equal(ht.to_numpy(Td), To)
    P = b["P"] * (1 + np.asfortranarray(rng.uniform(-0.01, 0.01, b["P"].shape)))
    Po, Pd = P.copy(order="F"), ht.from_numpy(P)
    orc.call("SetPressureBCs_dim", Po, b["wN2"], phc, p.Ptop, nx, ny, nz)
    api.SetPressureBCs_dim(ctx, Pd, ht.from_numpy(b["wN2"]), ht.from_numpy(phc), p.Pbot, p.Ptop)
    np.testing.assert_array_equal(ht.to_numpy(Pd), Po)
    # the x ghost (0, 3, 2) takes the pre-call value of the air cell (1, 3, 2), which the call resets to Ptop
    assert Po[0, 3, 2] == P[1, 3, 2] and Po[1, 3, 2] == p.Ptop != P[1, 3, 2]


def test_flux_and_residual_kernels(ctx, orc):
    b = setup()
    p = b["params"]
    nx, ny, nz = (s - 2 for s in b["T"].shape)
    rng = np.random.default_rng(10)
    k = [np.asfortranarray(rng.uniform(0.5, 2, s)) for s in ((nx + 1, ny, nz), (nx, ny + 1, nz), (nx, ny, nz + 1))]
    kd = [ht.from_numpy(a) for a in k]
    rfv = np.asfortranarray(rng.uniform(0.9, 1.1, (nx + 1, ny + 1, nz + 1)))
    q = [np.zeros(a.shape, order="F") for a in k]
    qd = [ht.zeros(*a.shape) for a in k]
    h = (1 / p.dx, 1 / p.dy, 1 / p.dz)
    orc.call("ComputeDarcyFlux", *q, rfv, *k, b["P"], p.g, *h, nx, ny, nz)
    api.ComputeDarcyFlux(ctx, *qd, ht.from_numpy(rfv), *kd, ht.from_numpy(b["P"]), p.g, *h)
    for a, bb in zip(qd, q):
        same(ht.to_numpy(a), bb)
    F, Fd = np.zeros((nx, ny, nz), order="F"), ht.zeros(nx, ny, nz)
    prf, prf0, PC = (np.asfortranarray(rng.uniform(0.5, 1.5, (nx, ny, nz))) for _ in range(3))
    orc.call("ResidualFluidPressure", F, b["phc2"], prf, prf0, PC, *q, 1.0, 3.0, *h, nx, ny, nz)
    api.ResidualFluidPressure(ctx, Fd, ht.from_numpy(b["phc2"]), ht.from_numpy(prf), ht.from_numpy(prf0),
                              ht.from_numpy(PC), *qd, 1.0, 3.0, *h)
    same(ht.to_numpy(Fd), F)
    T0 = np.asfortranarray(b["T"][1:-1, 1:-1, 1:-1] * 0.99)
    orc.call("ResidualTemperatureLinearised", F, b["T"], T0, prf, b["phc2"], PC, *q, 0.5, 1.0, 3.0, *h, nx, ny, nz)
    api.ResidualTemperatureLinearised(ctx, Fd, ht.from_numpy(b["T"]), ht.from_numpy(T0), ht.from_numpy(prf),
                                      ht.from_numpy(b["phc2"]), ht.from_numpy(PC), *qd, 0.5, 1.0, 3.0, *h)
    same(ht.to_numpy(Fd), F)
    V = [np.zeros(a.shape, order="F") for a in k]
    Vd = [ht.zeros(*a.shape) for a in k]
    orc.call("Init_vel_dim", *V, *q, rfv, nx, ny, nz)
    api.Init_vel_dim(ctx, *Vd, *qd, ht.from_numpy(rfv))
    for a, bb in zip(Vd, V):
        same(ht.to_numpy(a), bb)


@pytest.mark.parametrize("n", [(8, 9, 6), (24, 20, 12)])
def test_step_v18_matches_oracle(ctx, orc, n):
    """Three dimensional time steps (the steady initialisation, then transient
    steps with pluton insertion and WENO5-v2 sub-steps): the same thermal and
    Darcy iteration counts as the oracle, T, P and the Darcy velocities V
    within 1e-12 relative max-norm."""
    b = setup(n)
    nx, ny, nz = n
    V = [np.zeros(s, order="F") for s in ((nx + 1, ny, nz), (nx, ny + 1, nz), (nx, ny, nz + 1))]
    T, P = b["T"].copy(order="F"), b["P"].copy(order="F")
    Td, Pd = ht.from_numpy(T), ht.from_numpy(P)
    Vd = [ht.zeros(*v.shape) for v in V]
    phc, phv, wN, kmul = b["phc"], b["phv"], b["wN"], b["kmul"]
    args_d = (ht.from_numpy(phc), ht.from_numpy(phv), ht.from_numpy(wN), ht.from_numpy(kmul))
    p_o, p_d = b["params"], v18.box(*n, seed=3, nitout=50, tol=1e-9)["params"]
    inner = (slice(1, -1),) * 3
    for it in range(3):
        p_o.it = p_d.it = it
        s, st_t, st_p = orc.step_v18(T, P, phc, phv, wN, kmul, *V, p_o)
        assert s == 0
        gt, gp = api.step_v18(ctx, Td, Pd, *args_d, *Vd, p_d)
        assert gt.status == 0 and gp.status == 0
        assert (gt.iters, gp.iters) == (st_t.iters, st_p.iters), it
        assert p_d.n_adv == p_o.n_adv and p_d.dt == p_o.dt
        assert rel_err(ht.to_numpy(Td)[inner], T[inner]) <= 1e-12
        assert rel_err(ht.to_numpy(Pd)[inner], P[inner]) <= 1e-12
        for vd, v in zip(Vd, V):
            assert rel_err(ht.to_numpy(vd), v) <= 1e-12


@pytest.mark.parametrize("grid", [(250, 106, 3), (47, 31, 9)])
def test_set_initial_conditions_khaled(ctx, orc, grid):
    """Device SetInitialConditions_Khaled against the oracle: phases of cells
    and vertices, T and P identical; every phase present on the driver's grid;
    wN untouched."""
    from hydrothermal3d_gb300 import v18
    case = v18.khaled_case(*grid)
    nx, ny, nz = grid
    phc, phv = np.zeros((nx + 2, ny + 2, nz + 2), order="F"), np.zeros((nx + 1, ny + 1, nz + 1), order="F")
    T, P = np.zeros_like(phc, order="F"), np.zeros_like(phc, order="F")
    wN = np.asfortranarray(np.full((nx + 2, nz + 2), 0.25))
    orc.call("SetInitialConditions_Khaled", phc, phv, wN, ctypes.byref(case["geom"]), T, P, case["Tbot"],
             case["Ttop"], case["Pbot"], case["Ptop"], case["xmin"], case["ymin"], case["zmin"], case["xmax"],
             case["ymax"], case["zmax"], case["L"], nx, ny, nz)
    d = [ht.zeros(*a.shape) for a in (phc, phv, T, P)]
    wNd = ht.from_numpy(wN)
    api.SetInitialConditions_Khaled(ctx, d[0], d[1], wNd, case, d[2], d[3])
    for a, b in zip(d, (phc, phv, T, P)):
        np.testing.assert_array_equal(ht.to_numpy(a), b)
    np.testing.assert_array_equal(ht.to_numpy(wNd), wN)
    if grid == (250, 106, 3):
        assert set(np.unique(phc)) == {0.0, 1.0, 2.0, 3.0}
    inner = (slice(1, -1),) * 3
    assert T[inner].max() <= case["Tbot"] and T[inner].min() >= case["Ttop"] - 1e-12
