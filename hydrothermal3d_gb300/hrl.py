"""Problem set-up for the dimensionless Horton-Rogers-Lapwood (porous
convection) workload: the physics of Dimensionless/HydroThermal3D_Alban_v6.jl
in a unit cube, solved with DYREL.

Initial condition: T linear from Tbot = 1 (bottom, y = 0) to Ttop = 0 (top,
y = 1) at the cell centres (ghosts included), plus a seeded uniform
perturbation of amplitude ``amp`` on the inner cells; P = 0; uniform
conductivity and permeability (ktv = kfv = 1).

Boundary conditions (Alban_v6.jl:108-130, 153-159):
  thermal : x, z Neumann; y Dirichlet Tbot / Ttop
  Darcy   : all Neumann, buoyancy flux through top/bottom removed
            (KillNorthSouthFluxes!)
  WENO5   : W/E/B/F Neumann, S/N Dirichlet Tbot/Ttop
            (Dimensionless/kernels_HT3D.jl:164-177)
Time step: dt0 = min(dx,dy,dz)^2/6.1 (Dimensionless/HydroThermal3D_v7.jl:68),
then dt = dt_fact/6.1*min(dx,dy,dz)/max|V| after each step (v7.jl:220).
dt_fact defaults to 1: with v7's value 10 the next step's dt is set from a
velocity that the onset of convection then multiplies by ~30, the CFL number
reaches ~50 and WENO5/SSP-RK2 blows up within five steps (T leaves [0, 1]);
with 1 the onset peaks near CFL 7 and the run settles at CFL 0.17.
"""
import numpy as np

from . import abi

N, D = abi.BC_NEUMANN, abi.BC_DIRICHLET


def initial_fields(nx, ny, nz, seed=1, amp=1e-3, Tbot=1.0, Ttop=0.0, L=(1.0, 1.0, 1.0)):
    """Return numpy (Fortran-order) Tc_ex, Pc_ex, ktv, kfv for the HRL set-up."""
    Lx, Ly, Lz = L
    dy = Ly / ny
    yce = np.linspace(-dy / 2, Ly + dy / 2, ny + 2)
    T = np.empty((nx + 2, ny + 2, nz + 2), order="F")
    T[...] = (Tbot + (Ttop - Tbot) * yce / Ly)[None, :, None]
    rng = np.random.default_rng(seed)
    pert = rng.uniform(-amp, amp, size=(nz, ny, nx)).transpose(2, 1, 0)
    T[1:-1, 1:-1, 1:-1] += pert
    P = np.zeros((nx + 2, ny + 2, nz + 2), order="F")
    ktv = np.ones((nx + 1, ny + 1, nz + 1), order="F")
    kfv = np.ones((nx + 1, ny + 1, nz + 1), order="F")
    return T, P, ktv, kfv


def params(nx, ny, nz, Ra=1000.0, tol=1e-8, nitmax=10000, nitout=1000, dt_fact=1.0, weno_variant=abi.WENO_V1,
           L=(1.0, 1.0, 1.0), Tbot=1.0, Ttop=0.0, advection=True, dt_adapt=True, dt_max=0.0):
    Lx, Ly, Lz = L
    dx, dy, dz = Lx / nx, Ly / ny, Lz / nz
    p = abi.HrlParams()
    p.Ra, p.dx, p.dy, p.dz = Ra, dx, dy, dz
    p.dt = min(dx, dy, dz) ** 2 / 6.1
    p.Tbot, p.Ttop = Tbot, Ttop
    p.thermal_bc = abi.int6(N, N, D, D, N, N)
    p.thermal_val = abi.dbl6(0, 0, Tbot, Ttop, 0, 0)
    p.darcy_bc = abi.int6(N, N, N, N, N, N)
    p.darcy_val = abi.dbl6(0, 0, 0, 0, 0, 0)
    p.weno_bc = abi.int6(N, N, D, D, N, N)
    p.weno_val = abi.dbl6(0, 0, Tbot, Ttop, 0, 0)
    p.weno_variant = weno_variant
    p.kill_ns = 1
    p.dt_adapt = 1 if dt_adapt else 0
    p.advection = 1 if advection else 0
    p.dt_fact = dt_fact
    p.dt_max = dt_max
    p.thermal = abi.DyrelParams.reference(tol=tol, nitmax=nitmax, nitout=nitout)
    p.darcy = abi.DyrelParams.reference(tol=tol, nitmax=nitmax, nitout=nitout)
    return p


def ensemble(n_members=64, seed=4, nmin=31, nmax=95, ra=(100.0, 5000.0), log10k_sigma=0.25, corr_cells=4.0,
             dt_max=1e-3, **kw):
    """Members of the ensemble workload: per member, cells per axis drawn
    from U{nmin..nmax}, Ra log-uniform on [ra[0], ra[1]], an independent
    log-normal permeability kfv (log10 k ~ N(0, log10k_sigma) with a Gaussian
    correlation of corr_cells cells) and the HRL initial condition; ktv = 1.
    Returns a list of (Tc_ex, Pc_ex, ktv, kfv, HrlParams) with numpy fields.
    Extra keyword arguments go to params().

    The adapted dt is capped at dt_max: near the critical Rayleigh number the
    velocity stays small for many steps, the reference's rule lets dt grow
    without bound (to ~10^2 diffusion times), and convection then sets in
    within one step at a CFL number above 10, which WENO5/SSP-RK2 does not
    survive (a Ra = 118 member reached NaN at step 12 in FP64 as well)."""
    from .v18 import lognormal_field
    rng = np.random.default_rng(seed)
    out = []
    for m in range(n_members):
        nx, ny, nz = (int(v) for v in rng.integers(nmin, nmax + 1, size=3))
        Ra = float(np.exp(rng.uniform(np.log(ra[0]), np.log(ra[1]))))
        T, P, ktv, _ = initial_fields(nx, ny, nz, seed=int(rng.integers(1 << 30)))
        h = 1.0 / max(nx, ny, nz)
        g = lognormal_field((nx + 1, ny + 1, nz + 1), (1.0 / nx, 1.0 / ny, 1.0 / nz), mean=0.0, sigma=log10k_sigma,
                            corr=corr_cells * h, seed=int(rng.integers(1 << 30)))
        kfv = np.asfortranarray(10.0 ** g)
        out.append((T, P, ktv, kfv, params(nx, ny, nz, Ra=Ra, dt_max=dt_max, **kw)))
    return out


def lognormal_torch(shape, sigma=0.25, corr_cells=4.0, seed=5, device="cuda"):
    """10**g with g ~ N(0, sigma) correlated by a Gaussian of corr_cells cells:
    white noise filtered in Fourier space (torch, FP64, on `device`) and
    normalised to zero mean and unit variance before scaling."""
    import torch
    gen = torch.Generator(device=device)
    gen.manual_seed(seed)
    w = torch.randn(shape, generator=gen, dtype=torch.float64, device=device)
    k2 = 0.0
    for ax, n in enumerate(shape):
        f = torch.fft.fftfreq(n, dtype=torch.float64, device=device) * 2 * np.pi  # per cell
        sh = [1] * len(shape)
        sh[ax] = n
        k2 = k2 + f.reshape(sh) ** 2
    g = torch.fft.ifftn(torch.fft.fftn(w) * torch.exp(-k2 * corr_cells ** 2 / 4.0)).real
    del w
    g = (g - g.mean()) / g.std()
    return torch.pow(10.0, sigma * g)


def fault_slab_case(n=511, seed=5, Ra=1000.0, slab_factor=10.0, slab_cells=3, log10k_sigma=0.25, corr_cells=4.0,
                    dt_max=1e-3, device="cuda", **kw):
    """Large-grid HRL case: n^3 cells, log-normal background permeability
    (log10 k ~ N(0, log10k_sigma), Gaussian correlation of corr_cells cells),
    a vertical slab slab_cells cells wide at mid-x whose permeability is
    multiplied by slab_factor, and the HRL initial condition (perturbation
    amplitude 1e-3).  Built on `device`; returns column-major tensors
    (Tc_ex, Pc_ex, ktv, kfv) and the HrlParams."""
    import torch
    from . import api
    nx = ny = nz = n
    kw_t = dict(dtype=torch.float64, device=device)
    dy = 1.0 / ny
    yce = torch.arange(ny + 2, **kw_t) * dy - 0.5 * dy
    T = api.zeros(nx + 2, ny + 2, nz + 2, device=device)
    T.copy_((1.0 - yce)[None, :, None].expand(nx + 2, ny + 2, nz + 2))
    gen = torch.Generator(device=device)
    gen.manual_seed(seed + 1)
    T[1:-1, 1:-1, 1:-1] += (torch.rand((nx, ny, nz), generator=gen, **kw_t) * 2.0 - 1.0) * 1e-3
    P = api.zeros(nx + 2, ny + 2, nz + 2, device=device)
    ktv = api.ones(nx + 1, ny + 1, nz + 1, device=device)
    kfv = api.zeros(nx + 1, ny + 1, nz + 1, device=device)
    kfv.copy_(lognormal_torch((nx + 1, ny + 1, nz + 1), log10k_sigma, corr_cells, seed, device))
    c0 = nx // 2 - slab_cells // 2  # first slab cell; its vertices c0 .. c0 + slab_cells
    kfv[c0:c0 + slab_cells + 1] *= slab_factor
    return T, P, ktv, kfv, params(nx, ny, nz, Ra=Ra, dt_max=dt_max, **kw)


def bytes_per_iteration(nx, ny, nz, s):
    """Algorithmic bytes of one dimensionless DYREL pseudo-iteration:
    update {X, F0} (read+write) and read {kx, ky, kz, R, PC}: 9*N*s."""
    return 9 * nx * ny * nz * s


def bytes_per_advection(nx, ny, nz, s):
    """WENO5 SSP-RK2 over three axes: 7*N*s per axis."""
    return 21 * nx * ny * nz * s
