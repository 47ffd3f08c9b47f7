"""Known-answer tests that pin the oracle to the reference's own test script
and notebook (tools/TestAdvection.jl, notebooks/Gershgorin_TH3D.ipynb) and to
exact discrete properties of the scheme."""
import ctypes

import numpy as np

from hydrothermal3d_gb300 import abi


def test_linear_profile_is_discrete_steady_state(orc):
    """T = 1 - y with Dirichlet top/bottom and uniform k: div q = 0."""
    nx, ny, nz = 6, 9, 5
    dy = 1.0 / ny
    yce = np.linspace(-dy / 2, 1 + dy / 2, ny + 2)
    T = np.asfortranarray(np.broadcast_to((1.0 - yce)[None, :, None], (nx + 2, ny + 2, nz + 2)).copy())
    orc.call("SetFaceBCs", T, orc.int6(0, 0, 1, 1, 0, 0), orc.dbl6(0, 0, 1.0, 0.0, 0, 0), nx, ny, nz)
    kx, ky, kz = np.ones((nx + 1, ny, nz), order="F"), np.ones((nx, ny + 1, nz), order="F"), np.ones((nx, ny, nz + 1), order="F")
    qx, qy, qz = orc.zeros(nx + 1, ny, nz), orc.zeros(nx, ny + 1, nz), orc.zeros(nx, ny, nz + 1)
    orc.call("ComputeFlux", qx, qy, qz, kx, ky, kz, T, float(nx), float(ny), float(nz), nx, ny, nz)
    assert np.allclose(qy, 1.0, rtol=0, atol=1e-12)
    assert np.all(qx == 0) and np.all(qz == 0)
    F = orc.zeros(nx, ny, nz)
    orc.call("ResidualDiffusion", F, orc.zeros(nx, ny, nz), qx, qy, qz, float(nx), float(ny), float(nz), nx, ny, nz)
    assert np.max(np.abs(F)) <= 1e-10 * ny


def _residual(orc, T, kx, ky, kz, R, _dt, d):
    nx, ny, nz = (s - 2 for s in T.shape)
    qx, qy, qz = orc.zeros(nx + 1, ny, nz), orc.zeros(nx, ny + 1, nz), orc.zeros(nx, ny, nz + 1)
    orc.call("ComputeFlux", qx, qy, qz, kx, ky, kz, T, 1 / d[0], 1 / d[1], 1 / d[2], nx, ny, nz)
    F = orc.zeros(nx, ny, nz)
    orc.call("ResidualDiffusionTransient", F, T, R, qx, qy, qz, _dt, 1 / d[0], 1 / d[1], 1 / d[2], nx, ny, nz)
    return F


def test_gershgorin_is_row_sum_of_jacobian(orc):
    """notebooks/Gershgorin_TH3D.ipynb cell 2: G = sum |dF/dT_nb| over the 7-point stencil."""
    rng = np.random.default_rng(3)
    nx, ny, nz = 5, 4, 6
    d = (0.3, 0.5, 0.7)
    dt = 0.2
    kx, ky, kz = (np.asfortranarray(rng.uniform(0.5, 2, s)) for s in ((nx + 1, ny, nz), (nx, ny + 1, nz), (nx, ny, nz + 1)))
    T = np.asfortranarray(rng.uniform(0, 1, (nx + 2, ny + 2, nz + 2)))
    R = orc.zeros(nx, ny, nz)
    G, D = orc.zeros(nx, ny, nz), orc.zeros(nx, ny, nz)
    orc.call("GershgorinPoisson", G, D, np.ones((nx, ny, nz), order="F"), kx, ky, kz, 1.0, dt, *d, nx, ny, nz)
    F0 = _residual(orc, T, kx, ky, kz, R, 1 / dt, d)
    i, j, k = 2, 1, 3  # cell (0-based) whose row we check
    row = 0.0
    for (di, dj, dk) in ((0, 0, 0), (1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)):
        Tp = T.copy(order="F")
        Tp[i + 1 + di, j + 1 + dj, k + 1 + dk] += 1.0
        row += abs(_residual(orc, Tp, kx, ky, kz, R, 1 / dt, d)[i, j, k] - F0[i, j, k])
    assert abs(G[i, j, k] * D[i, j, k] - row) <= 1e-10 * row


def test_drhodp_is_pressure_derivative_of_rhof(orc):
    """notebooks/Gershgorin_TH3D.ipynb cell 4: dρdP_C = ∂ρf_C/∂p."""
    for Tc in (20.0, 150.0, 400.0):
        for p in (1e6, 5e7, 2e8):
            h = 1e3
            fd = (orc.law(5, Tc, p + h) - orc.law(5, Tc, p - h)) / (2 * h)
            an = orc.law(6, Tc, p)
            assert abs(fd - an) <= 1e-5 * abs(an)


def test_testadvection_gaussian_translation(orc):
    """tools/TestAdvection.jl:33-118: Gaussian 5exp(-r^2/0.1^2)+1 on a 122x122x3 grid,
    V = (1,1,0), C = 0.5, 50 steps of AdvectWithWeno5_v2; the peak must follow
    x0 + t V (the script prints the expected and actual peak positions)."""
    ncx = ncy = 16 * 8 - 6
    ncz = 3
    xmin, xmax, ymin, ymax, zmin, zmax = -1.0, 1.0, -1.0, 1.0, 0.0, 1.0
    Lx, Ly, Lz = xmax - xmin, ymax - ymin, zmax - zmin
    dx, dy, dz = Lx / ncx, Ly / ncy, Lz / ncz
    xce = np.linspace(xmin - dx / 2, xmax + dx / 2, ncx + 2)
    yce = np.linspace(ymin - dy / 2, ymax + dy / 2, ncy + 2)
    x0, y0, sx, sy = -Lx / 4, -Ly / 4, 0.1, 0.1
    T = np.asfortranarray(np.broadcast_to((5 * np.exp(-((xce[:, None] - x0) ** 2) / sx ** 2 - ((yce[None, :] - y0) ** 2) / sy ** 2) + 1.0)[:, :, None],
                                          (ncx + 2, ncy + 2, ncz + 2)).copy())
    Vx = np.ones((ncx + 1, ncy, ncz), order="F")
    Vy = np.ones((ncx, ncy + 1, ncz), order="F")
    Vz = np.zeros((ncx, ncy, ncz + 1), order="F")
    dt = 0.5 * min(dx, dy, dz) / 1.0
    types = orc.int6(0, 0, 1, 1, 0, 0)
    vals = orc.dbl6(0, 0, 1.0, 1.0, 0, 0)
    t = 0.0
    for it in range(50):
        t += dt
        orc.call("AdvectWithWeno5_v2", T, Vx, Vy, Vz, dt, 1 / dx, 1 / dy, 1 / dz, types, vals, ctypes.c_int(1), ncx, ncy, ncz)
        I = np.unravel_index(np.argmax(T[:, :, 1]), T[:, :, 1].shape)
        assert abs(x0 + t * 1.0 - xce[I[0]]) <= dx
        assert abs(y0 + t * 1.0 - yce[I[1]]) <= dy
    # the scheme keeps the solution bounded (no spurious growth)
    assert T[1:-1, 1:-1, 1:-1].max() <= 6.0 + 1e-6 and T[1:-1, 1:-1, 1:-1].min() >= 1.0 - 1e-2


def test_dyrel_parameters(orc):
    """h1, h2 and dtau from lambda_max exactly as Dimensional/HydroThermal3D_v18.jl:433-439."""
    nx = ny = nz = 4
    rng = np.random.default_rng(5)
    X = np.asfortranarray(rng.uniform(0, 1, (nx + 2,) * 3))
    k = [np.ones(s, order="F") for s in ((nx + 1, ny, nz), (nx, ny + 1, nz), (nx, ny, nz + 1))]
    R = orc.zeros(nx, ny, nz)
    F, F0 = orc.zeros(nx, ny, nz), orc.zeros(nx, ny, nz)
    prm = abi.DyrelParams.reference(nitout=1000)
    s, st = orc.dyrel_solve_dimless(X, R, *k, 0.0, 0.25, 0.25, 0.25, [0] * 6, [0.0] * 6, prm, F, F0, n_iter_fixed=1)
    lmax = st.lambda_max
    lmin = lmax / 500
    dtau = 2.0 / np.sqrt(lmax) * 0.99
    c = 2.0 * np.sqrt(lmin) * 0.5
    assert st.dtau == dtau
    assert st.h1 == (2 - c * dtau) / (2 + c * dtau) and st.h2 == 2 * dtau / (2 + c * dtau)
    # uniform k, Neumann: G/D = 2 (sum |offdiag| = diag)
    assert abs(lmax - 2.0) <= 1e-14


def test_weno5_mass_of_a_translated_blob(orc):
    """Advective-form WENO5 conserves the blob's mass to truncation error
    (Gaussian of the TestAdvection.jl set-up, uniform V, walls far away); the
    reference's v2 stencil quirk loses more than the fixed stencil."""
    ncx = ncy = 122
    ncz = 3
    dx = dy = 2.0 / ncx
    dz = 1.0 / ncz
    xce = np.linspace(-1 - dx / 2, 1 + dx / 2, ncx + 2)
    yce = np.linspace(-1 - dy / 2, 1 + dy / 2, ncy + 2)
    base = (5 * np.exp(-((xce[:, None] + 0.5) ** 2) / 0.01 - ((yce[None, :] + 0.5) ** 2) / 0.01) + 1.0)[:, :, None]
    Vx = np.ones((ncx + 1, ncy, ncz), order="F")
    Vy = np.ones((ncx, ncy + 1, ncz), order="F")
    Vz = np.zeros((ncx, ncy, ncz + 1), order="F")
    dt = 0.5 * min(dx, dy, dz)
    drift = {}
    for variant in (abi.WENO_V2_REF, abi.WENO_V2_FIXED):
        T = np.asfortranarray(np.broadcast_to(base, (ncx + 2, ncy + 2, ncz + 2)).copy())
        m0 = (T[1:-1, 1:-1, 1:-1] - 1).sum()
        for _ in range(50):
            orc.call("AdvectWithWeno5_v2", T, Vx, Vy, Vz, dt, 1 / dx, 1 / dy, 1 / dz, orc.int6(0, 0, 1, 1, 0, 0),
                     orc.dbl6(0, 0, 1.0, 1.0, 0, 0), ctypes.c_int(1 if variant == abi.WENO_V2_REF else 0), ncx,
                     ncy, ncz)
        drift[variant] = abs((T[1:-1, 1:-1, 1:-1] - 1).sum() - m0) / m0
    assert drift[abi.WENO_V2_FIXED] < 5e-3
    assert drift[abi.WENO_V2_FIXED] < drift[abi.WENO_V2_REF] < 1e-2


def test_geotherm_column_matches_1d_solve(orc):
    """Steady DYREL solve with y-varying k and source: x/z-invariant and equal
    to the exact 1-D solve of the same discrete operator."""
    from kat_cases import GEO_N, GEO_BC, geotherm_case, geotherm_exact, geotherm_params
    nx, ny, nz = GEO_N
    c = geotherm_case()
    X = np.zeros((nx + 2, ny + 2, nz + 2), order="F")
    F, F0 = orc.zeros(nx, ny, nz), orc.zeros(nx, ny, nz)
    s, st = orc.dyrel_solve_dimless(X, c["R"], c["kx"], c["ky"], c["kz"], 0.0, *c["d"], *GEO_BC, geotherm_params(),
                                    F, F0)
    assert s == 0
    col = X[1:-1, 1:-1, 1:-1]
    assert np.ptp(col, axis=(0, 2)).max() == 0.0
    Tex = geotherm_exact(c)
    assert np.abs(col - Tex[None, :, None]).max() <= 1e-12 * np.abs(Tex).max()


def test_hrl_onset_growth_factor(orc):
    """Horton-Rogers-Lapwood onset: below Ra = 4 pi^2 the mode decays, above
    it grows, each step by the linear factor (1 + dt Ra/2)/(1 + 2 pi^2 dt)."""
    from kat_cases import ONSET_N, ONSET_STEPS, onset_case, onset_factor
    n = ONSET_N
    for Ra in (20.0, 80.0):
        T, P, ktv, kfv, p, amplitude = onset_case(Ra)
        V = [np.zeros(s, order="F") for s in ((n + 1, n, n), (n, n + 1, n), (n, n, n + 1))]
        a = [amplitude(T[1:-1, 1:-1, 1:-1])]
        for _ in range(ONSET_STEPS):
            s, _, _ = orc.step_hrl(T, P, ktv, kfv, *V, p)
            assert s == 0
            a.append(amplitude(T[1:-1, 1:-1, 1:-1]))
        ratios = np.array(a[1:]) / np.array(a[:-1])
        G = onset_factor(Ra)
        assert np.all(np.abs(ratios - G) <= 5e-3 * G), (Ra, ratios, G)
        assert (a[-1] < a[0]) if Ra < 4 * np.pi ** 2 else (a[-1] > a[0])


def test_crustal_geotherm_benchmark_steady_state(orc):
    """Dimensional/Benchmarks/Geotherm_1D_weights.jl: the dimensional step's
    steady initialisation (it = 0) on the benchmark's column -- basal flux
    qmoho, immersed surface cell with weight wN, air at Tsurf, conductivity
    fixed from the initial 20 K/km profile -- equals the profile marched
    down from the surface with the flux qmoho through every rock face."""
    from kat_cases import GEO18_N, geotherm_v18_case, geotherm_v18_exact, geotherm_v18_ky
    nx, ny, nz = GEO18_N
    c = geotherm_v18_case()
    assert 0.0 < c["wN_value"] < 1.0
    ky = geotherm_v18_ky(orc, c)
    assert np.ptp(ky, axis=(0, 2)).max() <= 1e-15 * ky.max()  # the smoothing keeps a linear k(T(y)) per column
    T, P = c["T"].copy(order="F"), c["P"].copy(order="F")
    V = [np.zeros(s, order="F") for s in ((nx + 1, ny, nz), (nx, ny + 1, nz), (nx, ny, nz + 1))]
    s, st_t, _ = orc.step_v18(T, P, c["phc"], c["phv"], c["wN"], None, *V, c["params"])
    assert s == 0 and st_t.converged
    exact = geotherm_v18_exact(c, ky)
    got = T[1:-1, 1:c["js"] + 2, 1:-1]
    assert np.abs(got - exact).max() <= 1e-12 * np.abs(exact).max()
    # the steady profile is not the initial one: the basal flux and the surface rule shaped it
    T0 = c["T"][1:-1, 1:c["js"] + 2, 1:-1]
    assert np.abs(exact - T0).max() >= 1e-3 * np.abs(exact).max()
