"""Time loop of the dimensionless Horton-Rogers-Lapwood model around
ht3d_step_hrl, with the driver-side pieces of the reference's loops:

* the Nusselt number Nu = sum(qy[:,end,:]) / (Lx Lz) / (nx nz) of the thermal
  flux (Dimensionless/HydroThermal3D_Alban_v6.jl:345-348), evaluated on the
  temperature after each step (the fused step advects before returning; the
  reference evaluates it after the thermal solve of the step);
* one JSON line per step with the time, dt, Nu, the range of T and the two
  solves' statistics (iterations, residual norms, lambda_min/max, h1, h2) --
  the values the reference prints per check (Dimensional/HydroThermal3D_v18.jl:
  440-441, 463, 575-577) and the Nu/time series Alban writes (:500-505);
* restart files every nout steps and restart from one
  (Dimensional/HydroThermal3D_v18.jl:384-395, 579-588): Breakpoint%05d.h5 in
  the reference's HDF5 layout (ht3d_breakpoint_write_h5/read_h5), or the
  library's raw format (fmt="bin").

The state (T, P) is never modified outside ht3d_step_hrl: Nu is computed on a
copy, so a run with the driver is bit-identical to a bare loop of steps."""
import json
import os

import torch

from . import api, abi


def _stats(st):
    return {name: getattr(st, name) for name, _ in abi.DyrelStats._fields_}


class NusseltProbe:
    """Nu of a temperature field: face conductivities from the vertex field
    (InitThermal!), the thermal boundary conditions on a copy of T's ghosts
    (SetFaceBCs), ComputeFlux! and ht3d_Nusselt."""

    def __init__(self, ctx, nx, ny, nz):
        self.ctx = ctx
        z = api.zeros
        self.Rt = z(nx, ny, nz)
        self.kx, self.ky, self.kz = z(nx + 1, ny, nz), z(nx, ny + 1, nz), z(nx, ny, nz + 1)
        self.qx, self.qy, self.qz = z(nx + 1, ny, nz), z(nx, ny + 1, nz), z(nx, ny, nz + 1)
        self.T = z(nx + 2, ny + 2, nz + 2)
        self.n = (nx, ny, nz)

    def __call__(self, T, ktv, p):
        nx, ny, nz = self.n
        self.ctx.synchronize()        # T is final on the context's stream ...
        self.T.copy_(T)
        torch.cuda.synchronize()      # ... and the copy (torch's stream) before the library reads it
        api.InitThermal(self.ctx, self.Rt, self.kx, self.ky, self.kz, self.T, ktv, 1.0 / p.dt)
        api.SetFaceBCs(self.ctx, self.T, list(p.thermal_bc), list(p.thermal_val))
        api.ComputeFlux(self.ctx, self.qx, self.qy, self.qz, self.kx, self.ky, self.kz, self.T, 1.0 / p.dx,
                        1.0 / p.dy, 1.0 / p.dz)
        return api.Nusselt(self.ctx, self.qy, nx * p.dx, nz * p.dz)


def breakpoint_path(out_dir, it, fmt="h5"):
    return os.path.join(out_dir, f"Breakpoint{it:05d}.{fmt}")


def run_hrl(ctx, T, P, ktv, kfv, V, params, steps, precision=abi.MIXED, log=None, nout=0, out_dir=None,
            restart_from=0, time=0.0, fmt="h5"):
    """Steps it = restart_from + 1 .. restart_from + steps of the HRL model in
    place on the device fields T, P (ghosted) and V = (Vx, Vy, Vz).  log: a
    path (JSON lines appended) or None.  nout > 0 writes a restart file every
    nout steps into out_dir; restart_from > 0 first reads that step's file
    (T, P, time and dt).  Returns the list of per-step records."""
    nx, ny, nz = (int(s) - 2 for s in T.shape)
    if restart_from > 0:
        time, params.dt = api.breakpoint_read(ctx, breakpoint_path(out_dir, restart_from, fmt), T, P)
    probe = NusseltProbe(ctx, nx, ny, nz)
    records = []
    fh = open(log, "a") if log else None
    try:
        for it in range(restart_from + 1, restart_from + steps + 1):
            dt = params.dt
            st_t, st_d = api.step_hrl(ctx, T, P, ktv, kfv, *V, params, precision)
            time += dt
            ctx.synchronize()
            inner = T[1:-1, 1:-1, 1:-1]
            rec = {"it": it, "time": time, "dt": dt, "Nu": probe(T, ktv, params),
                   "T_min": float(inner.min()), "T_max": float(inner.max()),
                   "thermal": _stats(st_t), "darcy": _stats(st_d)}
            records.append(rec)
            if fh:
                fh.write(json.dumps(rec) + "\n")
                fh.flush()
            if nout > 0 and it % nout == 0:
                api.breakpoint_write(ctx, breakpoint_path(out_dir, it, fmt), T, P, time, params.dt)
    finally:
        if fh:
            fh.close()
    return records
