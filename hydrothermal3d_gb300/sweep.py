"""Standalone WENO5 sweep workload: a temperature blob advected by a
discretely divergence-free velocity on the staggered grid.

The velocity is the discrete curl of a vector potential A stored on the cell
edges (Ax on x-edges at (xc, y, z), Ay on y-edges at (x, yc, z), Az on
z-edges at (x, y, zc)):

    Vx = dAz/dy - dAy/dz   (x-faces)
    Vy = dAx/dz - dAz/dx   (y-faces)
    Vz = dAy/dx - dAx/dy   (z-faces)

with one-cell differences, so the discrete divergence of every cell
(Vx[i+1]-Vx[i])/dx + ... vanishes identically (up to rounding).  Each
component of A is a sum of seeded modes sin(l pi x) sin(m pi y) sin(n pi z)
(integer l, m, n in 1..4): A vanishes on the walls, so does the normal
velocity.  The velocity is scaled to max |V| = vmax.

Arrays are built with torch on any device (the 511^3 case is built on the
GPU) and returned in the library's column-major layout.
"""
import numpy as np
import torch

from . import api


def _modes(n_modes, seed):
    """Per component of A: n_modes ((l, m, n), amplitude) pairs."""
    rng = np.random.default_rng(seed)
    return [[(tuple(int(v) for v in rng.integers(1, 5, size=3)), float(rng.normal())) for _ in range(n_modes)]
            for _ in range(3)]


def _field(modes, xs, ys, zs):
    """sum over modes of a * sin(l pi x) sin(m pi y) sin(n pi z) on the tensor grid xs x ys x zs."""
    out = None
    for (l, m, n), a in modes:
        t = a * torch.sin(l * np.pi * xs)[:, None, None] * torch.sin(m * np.pi * ys)[None, :, None] * \
            torch.sin(n * np.pi * zs)[None, None, :]
        out = t if out is None else out + t
    return out


def curl_velocity(nx, ny, nz, n_modes=8, seed=6, vmax=1.0, device="cuda", dtype=torch.float64):
    """(Vx, Vy, Vz) on the faces of the unit cube, column-major, max |V| = vmax."""
    modes = _modes(n_modes, seed)
    kw = dict(dtype=torch.float64, device=device)
    dx, dy, dz = 1.0 / nx, 1.0 / ny, 1.0 / nz
    xn, yn, zn = (torch.arange(n + 1, **kw) * h for n, h in ((nx, dx), (ny, dy), (nz, dz)))
    xc, yc, zc = (torch.arange(n, **kw) * h + 0.5 * h for n, h in ((nx, dx), (ny, dy), (nz, dz)))
    Ax = _field(modes[0], xc, yn, zn)  # (nx, ny+1, nz+1)
    Ay = _field(modes[1], xn, yc, zn)  # (nx+1, ny, nz+1)
    Az = _field(modes[2], xn, yn, zc)  # (nx+1, ny+1, nz)
    Vx = (Az[:, 1:, :] - Az[:, :-1, :]) / dy - (Ay[:, :, 1:] - Ay[:, :, :-1]) / dz  # (nx+1, ny, nz)
    Vy = (Ax[:, :, 1:] - Ax[:, :, :-1]) / dz - (Az[1:, :, :] - Az[:-1, :, :]) / dx  # (nx, ny+1, nz)
    Vz = (Ay[1:, :, :] - Ay[:-1, :, :]) / dx - (Ax[:, 1:, :] - Ax[:, :-1, :]) / dy  # (nx, ny, nz+1)
    del Ax, Ay, Az
    s = vmax / max(float(Vx.abs().max()), float(Vy.abs().max()), float(Vz.abs().max()))
    out = []
    for V in (Vx, Vy, Vz):
        d = api.zeros(*V.shape, dtype=dtype, device=device)
        d.copy_(V * s)
        out.append(d)
    return tuple(out)


def divergence(Vx, Vy, Vz):
    """Discrete divergence of every cell (logical (nx, ny, nz) tensor)."""
    nx, ny, nz = Vx.shape[0] - 1, Vy.shape[1] - 1, Vz.shape[2] - 1
    return ((Vx[1:] - Vx[:-1]) * nx + (Vy[:, 1:] - Vy[:, :-1]) * ny + (Vz[:, :, 1:] - Vz[:, :, :-1]) * nz)


def blob(nx, ny, nz, width=0.1, centre=(0.5, 0.35, 0.5), device="cuda", dtype=torch.float64):
    """Ghosted temperature (nx+2, ny+2, nz+2): a Gaussian blob of unit height on
    a zero background, evaluated at the cell centres (ghosts included)."""
    kw = dict(dtype=torch.float64, device=device)
    c = [(torch.arange(n + 2, **kw) - 0.5) / n for n in (nx, ny, nz)]
    g = [torch.exp(-((ci - x0) / width) ** 2) for ci, x0 in zip(c, centre)]
    T = g[0][:, None, None] * g[1][None, :, None] * g[2][None, None, :]
    d = api.zeros(nx + 2, ny + 2, nz + 2, dtype=dtype, device=device)
    d.copy_(T)
    return d


def cfl_dt(nx, ny, nz, vmax=1.0, cfl=0.5):
    """Advection time step at the given CFL number."""
    return cfl * min(1.0 / nx, 1.0 / ny, 1.0 / nz) / vmax


def bytes_per_sweep(nx, ny, nz, s):
    """Algorithmic bytes of one SSP-RK2 sweep over three axes: 7 N s per axis."""
    return 21 * nx * ny * nz * s
