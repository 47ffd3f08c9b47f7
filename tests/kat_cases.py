"""Known-answer cases of the scheme's physics, shared by the oracle (CPU) and
GPU tests:

* a y-column geotherm: steady diffusion with y-varying conductivity and
  source, Dirichlet top/bottom, x/z Neumann -- the 3-D DYREL solution must be
  x/z-invariant and equal the exact 1-D solve of the same discrete operator;
* the Horton-Rogers-Lapwood onset (Dimensionless/HydroThermal3D_Alban_v6.jl
  set-up): the mode cos(pi x) sin(pi y) of the unit box has critical
  Ra = 4 pi^2; with implicit diffusion and the mode's Darcy velocity
  Vy = Ra A / 2 each time step multiplies its amplitude by
  (1 + dt Ra / 2) / (1 + 2 pi^2 dt)."""
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
