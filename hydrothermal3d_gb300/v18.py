"""Set-up of the dimensional workload (the kernels and driver logic of
Dimensional/HydroThermal3D_v18.jl) on a synthetic box.

scaling() restates `scaling`/`scale_me!` (Dimensional/kernels_HT3D_dimensional.jl:3-36)
with the v18 characteristic values (T 500 K, V 1e-9 m/s, L 700 m, eta 1e10 Pa s).

box() builds the benchmark box: x 10 km, y (vertical) 10 km below the surface
at y = 0, z 5 km; T linear from T_bot to T_top; hydrostatic pressure; crust
everywhere with the top ghost row as air (phase 1, held at T_top / P_top);
permeability log10 k ~ N(mean, sigma) with a Gaussian correlation length,
built on the host in FP64 from seeded white noise filtered by FFT.  The
reference's depth law kF(y) = 5e-16 exp(y/delta) is neutralised (delta -> inf)
and the field enters ComputeHydroConductivity as the vertex multiplier kmul.
"""
import math

import numpy as np

from . import abi


def scaling(T=500.0, V=1e-9, L=700.0, eta=1e10):
    s = dict(T=T, V=V, L=L, eta=eta)
    s["t"] = L / V
    s["a"] = V / s["t"]
    s["eps"] = 1.0 / s["t"]
    s["sigma"] = eta / s["t"]
    s["m"] = s["sigma"] * L * s["t"] ** 2
    s["rho"] = s["m"] / L ** 3
    s["F"] = s["m"] * L / s["t"] ** 2
    s["J"] = s["m"] * L ** 2 / s["t"] ** 2
    s["W"] = s["J"] / s["t"]
    s["C"] = s["J"] / s["m"] / T
    s["kt"] = s["W"] / L / T
    s["kf"] = L ** 2
    return s


def lognormal_field(shape, spacing, mean=-15.0, sigma=0.5, corr=500.0, seed=2):
    """log10 k with a Gaussian covariance of length `corr` (m), FFT-filtered
    white noise normalised to the requested mean and standard deviation."""
    rng = np.random.default_rng(seed)
    w = rng.standard_normal(shape)
    k2 = 0.0
    for ax, (n, h) in enumerate(zip(shape, spacing)):
        f = np.fft.fftfreq(n, d=h) * 2 * np.pi
        sh = [1] * len(shape)
        sh[ax] = n
        k2 = k2 + (f.reshape(sh)) ** 2
    g = np.real(np.fft.ifftn(np.fft.fftn(w) * np.exp(-k2 * corr ** 2 / 4.0)))
    g = (g - g.mean()) / (g.std() if g.std() > 0 else 1.0)
    return mean + sigma * g


def box(nx, ny, nz, Lx=10e3, Ly=10e3, Lz=5e3, T_bot_C=600.0, T_top_C=20.0, seed=2, log10k_mean=-15.0,
        log10k_sigma=0.5, corr=500.0, tol=1e-10, nitout=1000, nitmax=10000, dt_s=1e11, cfl_adv=0.5,
        weno_variant=abi.WENO_V2_REF):
    sc = scaling()
    L = sc["L"]
    xmin, xmax = 0.0, Lx / L
    ymin, ymax = -Ly / L, 0.0
    zmin, zmax = 0.0, Lz / L
    dx, dy, dz = (xmax - xmin) / nx, (ymax - ymin) / ny, (zmax - zmin) / nz
    Ttop = (T_top_C + 273.15) / sc["T"]
    Tbot = (T_bot_C + 273.15) / sc["T"]
    Ptop = 1e5 / sc["sigma"]
    g = -9.81 / (L / sc["t"] ** 2)
    rho_w = 1000.0 / sc["rho"]
    Pbot = Ptop - rho_w * g * (ymax - ymin)
    yce = np.linspace(ymin - dy / 2, ymax + dy / 2, ny + 2)
    T = np.empty((nx + 2, ny + 2, nz + 2), order="F")
    T[...] = (Ttop + (Ttop - Tbot) * (yce - ymax) / (ymax - ymin))[None, :, None]
    P = np.empty((nx + 2, ny + 2, nz + 2), order="F")
    P[...] = (Ptop - rho_w * g * (ymax - yce))[None, :, None]
    phc = np.zeros((nx + 2, ny + 2, nz + 2), order="F")
    phc[:, -1, :] = 1.0  # air above the surface
    T[:, -1, :] = Ttop
    P[:, -1, :] = Ptop
    phv = np.zeros((nx + 1, ny + 1, nz + 1), order="F")
    wN = np.full((nx + 2, nz + 2), 0.5, order="F")
    lk = lognormal_field((nx + 1, ny + 1, nz + 1), (dx * L, dy * L, dz * L), log10k_mean, log10k_sigma, corr, seed)
    kmul = np.asfortranarray(10.0 ** lk / 5e-16)
    # impermeable basement: the reference's bottom pressure rule P[ghost] = P[inner]
    # is an outflow boundary under gravity; zero permeability on the bottom vertex
    # row makes the bottom face (whose ky averages only that row) no-flow
    kmul[:, 0, :] = 0.0
    # basal heat flux consistent with the initial gradient and the rock conductivity at the base
    kT_base = 3.1138 - 0.0023 * (Tbot * sc["T"])
    qyS_SI = kT_base * (T_bot_C - T_top_C) / Ly
    p = abi.V18Params()
    p.dx, p.dy, p.dz, p.ymin = dx, dy, dz, ymin
    p.dt = dt_s / sc["t"]
    p.time = 0.0
    p.phi_i, p.k_fact, p.delta, p.g, p.Qt = 1e-2, 50.0, 1e30 / L, g, 0.0
    p.qyS = qyS_SI / (sc["W"] / L ** 2)
    p.Ttop, p.Tbot, p.Ptop, p.Pbot = Ttop, Tbot, Ptop, Pbot
    p.T_pluton = (700.0 + 273.15) / sc["T"]
    p.C_adv = cfl_adv * 6.1
    p.sc_T, p.sc_L, p.sc_t, p.sc_eta = sc["T"], sc["L"], sc["t"], sc["eta"]
    p.sc_sigma, p.sc_rho, p.sc_C, p.sc_kt = sc["sigma"], sc["rho"], sc["C"], sc["kt"]
    p.it, p.thermal, p.hydro, p.advection, p.dt_constant = 0, 1, 1, 1, 1
    p.weno_variant = weno_variant
    # relative tolerance only: in the reference's scaled units an absolute norm
    # of 1e-10 is reached long before convergence (v18 itself uses 1e-18)
    p.thermal_dyrel = abi.DyrelParams.reference(tol=tol, nitmax=nitmax, nitout=nitout,
                                                norm_scale=sc["rho"] * sc["C"] * sc["T"] / sc["t"])
    p.thermal_dyrel.tol_abs = 0.0
    p.darcy_dyrel = abi.DyrelParams.reference(tol=tol, nitmax=nitmax, nitout=nitout, norm_scale=sc["rho"] / sc["t"])
    p.darcy_dyrel.tol_abs = 0.0
    return dict(T=T, P=P, phc=phc, phv=phv, wN=wN, kmul=kmul, params=p)


def bytes_per_iteration(nx, ny, nz, s=8):
    """Algorithmic bytes of one dimensional pseudo-iteration: thermal updates
    {T, F0} and reads {kx, ky, kz, T0, rhoC, PC} + phase (1 B): 10 N s + N;
    Darcy updates {P, F0} and reads {kx, ky, kz, T, phirhof0, rhof(y-face), PC}
    + phase: 11 N s + N.  Returns (thermal, darcy)."""
    N = nx * ny * nz
    return 10 * N * s + N, 11 * N * s + N


def _slope(x1, x2, y1, y2):
    """a(x1, x2, y1, y2) of v18.jl:40: slope of the line through two points."""
    return (y1 - y2) / (x1 - x2)


def _intercept(x1, x2, y1, y2):
    """b(x1, x2, y1, y2) of v18.jl:41: its intercept."""
    return y1 - x1 * (y1 - y2) / (x1 - x2)


def khaled_case(nx=250, ny=106, nz=3):
    """The detachment-fault model of the v18 driver (Dimensional/HydroThermal3D_v18.jl:162-287):
    domain, boundary values and the geometry of the main detachment, three
    secondary faults and the topography, in scaled units.  Returns a dict of
    the arguments of SetInitialConditions_Khaled.  The default grid is the
    driver's fact = 8 grid (ncx = 8*32-6, ncy = 8*14-6, ncz = 3); zmin is the
    driver's -25 m as written there."""
    sc = scaling()
    L = sc["L"]
    # corner points of each wedge: three lines (top, bottom, closing edge), v18.jl:184-233
    corners = {
        "fault": ((75.8e3, 31498.437753425103, 3e3, -16897.187956165293),
                  (32000.0, 77e3, -17800.0, 3e3),
                  (32000.0, 31498.437753425103, -17800.0, -16897.187956165293)),
        "fault1": ((59.5e3, 62.5e3, 0e3, -3e3), (61.8e3, 58.8e3, -3e3, 0e3), (62.5e3, 61.8e3, -3e3, -3e3)),
        "fault2": ((48.5e3, 54.5e3, 0e3, -7e3), (53.8e3, 47.8e3, -7e3, 0e3), (54.5e3, 53.8e3, -7e3, -7e3)),
        "fault3": ((36.8e3, 46.8e3, 0e3, -10.5e3), (46e3, 36e3, -10.5e3, 0e3), (46.8e3, 46e3, -10.5e3, -10.5e3)),
    }
    g = abi.KhaledGeom()
    g.y_plateau = 1.5e3 / L
    sx1, sx2, sy1, sy2 = 32000.0 / L, 69397.54576150524 / L, -17800.0 / L, 0.0 / L
    g.surf_a1, g.surf_b1 = _slope(sx1, sx2, sy1, sy2), _intercept(sx1, sx2, sy1, sy2)
    for f, name in enumerate(("fault", "fault1", "fault2", "fault3")):
        for e, (x1, x2, y1, y2) in enumerate(corners[name]):
            x1, x2, y1, y2 = x1 / L, x2 / L, y1 / L, y2 / L
            g.fault[f][2 * e] = _slope(x1, x2, y1, y2)
            g.fault[f][2 * e + 1] = _intercept(x1, x2, y1, y2)
    Ttop = 293.15 / sc["T"]
    Ptop = 1e5 / sc["sigma"]
    return dict(geom=g, Tbot=Ttop + 600.0 / sc["T"], Ttop=Ttop, Pbot=Ptop + 294e6 / sc["sigma"], Ptop=Ptop,
                xmin=30e3 / L, ymin=-30e3 / L, zmin=-25.0 / L, xmax=100e3 / L, ymax=5e3 / L, zmax=25e3 / L, L=L,
                nx=nx, ny=ny, nz=nz)
