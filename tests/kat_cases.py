"""Known-answer cases of the scheme's physics, shared by the oracle (CPU) and
GPU tests:

* a y-column geotherm: steady diffusion with y-varying conductivity and
  source, Dirichlet top/bottom, x/z Neumann -- the 3-D DYREL solution must be
  x/z-invariant and equal the exact 1-D solve of the same discrete operator;
* the Horton-Rogers-Lapwood onset (Dimensionless/HydroThermal3D_Alban_v6.jl
  set-up): the mode cos(pi x) sin(pi y) of the unit box has critical
  Ra = 4 pi^2; with implicit diffusion and the mode's Darcy velocity
  Vy = Ra A / 2 each time step multiplies its amplitude by
  (1 + dt Ra / 2) / (1 + 2 pi^2 dt);
* the reference's own 1-D crustal geotherm benchmark
  (Dimensional/Benchmarks/Geotherm_1D_weights.jl): a column from -30 km to
  +10 km in 26 cells, air above the surface (held at Tsurf), the
  immersed-surface cell (phase -1, weight wN) below it, a basal heat flux
  qmoho through the bottom ghost and conductivity fixed from the initial
  20 K/km profile.  At steady state the flux through every rock face equals
  qmoho; the immersed rule wN T_imm + (1 - wN) T_below = Tsurf then fixes
  the profile, marched down face by face: T_below = Tsurf + wN qmoho /
  (k/dy), T_{j-1} = T_j + qmoho / (k_{j-1/2}/dy).  The dimensional step's
  steady initialisation (it = 0) on this column must reproduce it."""
import numpy as np

from hydrothermal3d_gb300 import abi, hrl

# --------------------------------------------------------------- geotherm
GEO_N = (3, 24, 2)
GEO_BC = ([0, 0, 1, 1, 0, 0], [0.0, 0.0, 1.0, 0.0, 0.0, 0.0])  # Tbot = 1, Ttop = 0


def geotherm_case():
    nx, ny, nz = GEO_N
    dy = 1.0 / ny
    yf = np.arange(ny + 1) * dy
    yc = (np.arange(ny) + 0.5) * dy
    k_y = 1.0 + 0.5 * np.sin(3 * yf)
    R_y = -2.0 * np.cos(2 * yc)
    kx = np.ones((nx + 1, ny, nz), order="F")
    kz = np.ones((nx, ny, nz + 1), order="F")
    ky = np.asfortranarray(np.broadcast_to(k_y[None, :, None], (nx, ny + 1, nz)).copy())
    R = np.asfortranarray(np.broadcast_to(R_y[None, :, None], (nx, ny, nz)).copy())
    return dict(kx=kx, ky=ky, kz=kz, R=R, k_y=k_y, R_y=R_y, d=(1.0 / nx, dy, 1.0 / nz))


def geotherm_exact(c):
    """Exact solution of the 1-D discrete problem F(T) = 0 with
    F_j = R_j + (q_{j+1} - q_j)/dy, q_j = -k_j (T_j - T_{j-1})/dy and
    Dirichlet ghosts 2 v - inner (F is affine: assemble and solve)."""
    Tbot, Ttop = GEO_BC[1][2], GEO_BC[1][3]
    k_y, R_y, dy = c["k_y"], c["R_y"], c["d"][1]
    ny = R_y.size

    def F(T):
        g = np.concatenate(([2 * Tbot - T[0]], T, [2 * Ttop - T[-1]]))
        q = -k_y * (g[1:] - g[:-1]) / dy
        return R_y + (q[1:] - q[:-1]) / dy

    b = F(np.zeros(ny))
    A = np.stack([F(np.eye(ny)[m]) - b for m in range(ny)], axis=1)
    return np.linalg.solve(A, -b)


def geotherm_params():
    return abi.DyrelParams.reference(tol=1e-13, nitout=100, nitmax=200000)


# ------------------------------------------------------------------ onset
ONSET_N, ONSET_DT, ONSET_STEPS, ONSET_AMP = 16, 0.005, 8, 1e-3


def onset_case(Ra):
    n = ONSET_N
    T, P, ktv, kfv = hrl.initial_fields(n, n, n, seed=1, amp=0.0)
    xc = (np.arange(n) + 0.5) / n
    mode = np.cos(np.pi * xc)[:, None, None] * np.sin(np.pi * xc)[None, :, None] * np.ones((1, 1, n))
    T[1:-1, 1:-1, 1:-1] += ONSET_AMP * mode
    p = hrl.params(n, n, n, Ra=Ra, tol=1e-10, nitout=100, nitmax=20000, dt_max=ONSET_DT)
    p.dt = ONSET_DT
    cond = np.broadcast_to((1.0 - xc)[None, :, None], (n, n, n))
    amplitude = lambda Tin: float(((Tin - cond) * mode).sum() / (mode * mode).sum())
    return T, P, ktv, kfv, p, amplitude


def onset_factor(Ra, dt=ONSET_DT):
    return (1.0 + dt * Ra / 2.0) / (1.0 + 2.0 * np.pi ** 2 * dt)


# ------------------------------------------------- crustal geotherm (v18)
GEO18_N = (3, 26, 3)  # ny = 4*8-6 cells, as the benchmark's ncy
GEO18_SURF = 500.0    # m; off the cell centres so the immersed weight is fractional


def geotherm_v18_case():
    """The benchmark's column in the v18 step's scaled units: returns the
    ghosted T (initial 20 K/km profile everywhere, air included), P, phc,
    phv, wN and V18Params for a steady thermal solve only (it = 0, no Darcy
    solve, no advection)."""
    from hydrothermal3d_gb300 import v18
    nx, ny, nz = GEO18_N
    sc = v18.scaling()
    L = sc["L"]
    ymin, ymax = -30e3, 10e3
    Tsurf, qmoho, phi_i = 293.15, 37e-3, 1e-2
    dy_si = (ymax - ymin) / ny
    yce = np.linspace(ymin - dy_si / 2, ymax + dy_si / 2, ny + 2)
    tiny = 1e-9
    ph_y = np.zeros(ny + 2)
    ph_y[yce > GEO18_SURF - tiny] = 1.0
    ph_y[(yce > GEO18_SURF - tiny) & (yce < GEO18_SURF - tiny + 1.5 * dy_si)] = -1.0
    ind = int(np.flatnonzero(ph_y == -1.0)[0])
    wN = 1.0 - (yce[ind] - GEO18_SURF) / dy_si
    ex = (nx + 2, ny + 2, nz + 2)
    T = np.asfortranarray(np.broadcast_to(((-yce * 20e-3 + Tsurf) / sc["T"])[None, :, None], ex).copy())
    P = np.asfortranarray(np.full(ex, 1e5 / sc["sigma"]))
    phc = np.asfortranarray(np.broadcast_to(ph_y[None, :, None], ex).copy())
    phv = np.zeros((nx + 1, ny + 1, nz + 1), order="F")
    wN2 = np.full((nx + 2, nz + 2), wN, order="F")
    p = v18.box(nx, ny, nz, tol=1e-13, nitout=100, nitmax=400000)["params"]
    p.dy, p.ymin = dy_si / L, ymin / L
    p.phi_i, p.Qt = phi_i, 0.0
    p.qyS = qmoho / (sc["W"] / L ** 2)
    p.Ttop = Tsurf / sc["T"]
    p.it, p.thermal, p.hydro, p.advection = 0, 1, 0, 0
    return dict(T=T, P=P, phc=phc, phv=phv, wN=wN2, params=p, js=ind - 1, wN_value=wN)


def geotherm_v18_exact(c, ky):
    """Steady profile of ex cells 1..js+1 (rock, then the immersed cell) of
    every (i, k) column from the face conductivities ky (nx, ny+1, nz) the
    step uses: the flux through every rock face equals qyS."""
    p, js, wN = c["params"], c["js"], c["wN_value"]
    nx, _, nz = GEO18_N
    _dy = 1.0 / p.dy
    T = np.zeros((nx, js + 2, nz))
    for i in range(nx):
        for k in range(nz):
            T[i, js, k] = p.Ttop + wN * p.qyS / (_dy * ky[i, js, k])
            T[i, js + 1, k] = T[i, js, k] - p.qyS / (_dy * ky[i, js, k])
            for J in range(js, 1, -1):
                T[i, J - 1, k] = T[i, J, k] + p.qyS / (_dy * ky[i, J - 1, k])
    return T[:, 1:, :]  # ex cells 1 .. js+1


def geotherm_v18_ky(orc, c):
    """Face conductivities of the step's thermal solve, from the oracle's
    granular kernels on the initial T: ComputeThermalConductivity, the
    vertex -> cell -> vertex smoothing, InitConductivity."""
    p = c["params"]
    nx, ny, nz = GEO18_N
    kv = np.zeros((nx + 1, ny + 1, nz + 1), order="F")
    orc.call("ComputeThermalConductivity", kv, c["T"], c["phv"], p.phi_i, p.sc_kt, p.sc_T, nx, ny, nz)
    kc = np.zeros((nx, ny, nz), order="F")
    orc.call("SmoothConductivityV2C", kc, kv, nx, ny, nz)
    orc.call("SmoothConductivityC2V", kv, kc, nx, ny, nz)
    kx, ky, kz = (np.zeros(s, order="F") for s in ((nx + 1, ny, nz), (nx, ny + 1, nz), (nx, ny, nz + 1)))
    orc.call("InitConductivity", kx, ky, kz, kv, nx, ny, nz)
    return ky

