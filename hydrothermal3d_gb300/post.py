"""Output diagnostics workload: the v18 driver's VTK output step
(Dimensional/HydroThermal3D_v18.jl:664-686) on synthetic fields, run either as
the reference's ten kernels or as one fused ht3d_postprocess_fields pass."""
import torch

from . import api, abi

# dimensional scales and constants of the v18 driver's order of magnitude
PARAMS = dict(phi0=0.01, scale_T=600.0, scale_sigma=1e8, scale_V=1e-9, scale_L=1e3, k_fact=100.0, ymin=-30.0,
              dy=0.25, delta=2.0)


def device_case(nx, ny, nz, seed=0):
    """Seeded device fields: phases (0 crust, 2 fault, 3 pluton, -1 immersed,
    1 air in the top 5 % of the rows), T in [300, 900] K and P in
    [0.1, 300] MPa after scaling, face velocities in [-1, 1] (times scale_V)."""
    g = torch.Generator(device="cuda").manual_seed(seed)
    ex = (nx + 2, ny + 2, nz + 2)
    codes = torch.tensor([0.0, 0.0, 0.0, 2.0, 3.0, -1.0], dtype=torch.float64, device="cuda")
    phc = api.zeros(*ex)
    phc.copy_(codes[torch.randint(0, codes.numel(), ex, generator=g, device="cuda")])
    phc[:, ny + 2 - max(1, (ny + 2) // 20):, :] = 1.0
    u = lambda shape, lo, hi: api.zeros(*shape).uniform_(lo, hi, generator=g)
    return dict(phc=phc, T=u(ex, 0.5, 1.5), P=u(ex, 1e-3, 3.0), Vx=u((nx + 1, ny, nz), -1, 1),
                Vy=u((nx, ny + 1, nz), -1, 1), Vz=u((nx, ny, nz + 1), -1, 1))


def outputs(nx, ny, nz):
    return {k: api.zeros(nx, ny, nz) for k in abi.POST_FIELDS}


def run_separate(ctx, d, o, p=PARAMS):
    """The driver's sequence of ten diagnostic kernels."""
    api.Phase(ctx, o["phase"], d["phc"])
    api.Pressure(ctx, o["pressure"], d["P"], d["phc"], p["scale_sigma"])
    api.Temperature(ctx, o["temperature"], d["T"], d["phc"], p["scale_T"])
    api.Velocity(ctx, o["vx"], o["vy"], o["vz"], d["Vx"], d["Vy"], d["Vz"], d["phc"], p["scale_V"])
    api.EffectiveThermalConductivity(ctx, o["k_thermal"], d["T"], p["phi0"], d["phc"], p["scale_T"])
    api.Permeability(ctx, o["permeability"], p["k_fact"], p["ymin"], p["dy"], d["phc"], p["delta"], p["scale_L"])
    api.FluidDensity(ctx, o["density"], d["T"], d["P"], d["phc"], p["scale_T"], p["scale_sigma"])
    api.Viscosity(ctx, o["viscosity"], d["T"], d["phc"], p["scale_T"])
    api.Peclet(ctx, o["peclet"], d["T"], d["P"], d["Vx"], d["Vy"], d["Vz"], d["phc"], p["phi0"], p["scale_T"],
               p["scale_sigma"], p["scale_V"], p["scale_L"])
    api.EffectiveHeatCapacity(ctx, o["heat_capacity"], d["T"], d["P"], d["phc"], p["phi0"], p["scale_T"],
                              p["scale_sigma"], 1.0, 1.0)


def run_fused(ctx, d, o, p=PARAMS):
    api.postprocess_fields(ctx, o, d["T"], d["P"], d["Vx"], d["Vy"], d["Vz"], d["phc"], **p)


def bytes_fused(nx, ny, nz):
    """Algorithmic bytes of one fused pass: phc, T, P and the three face
    velocities read once (one value per cell each), twelve outputs written."""
    return 18 * 8 * nx * ny * nz


def bytes_separate(nx, ny, nz):
    """Algorithmic bytes of the ten kernels: Phase 2, Pressure 3, Temperature 3,
    Velocity 7, k_eff 3, permeability 2, density 4, viscosity 3, Peclet 7,
    heat capacity 3 arrays of one value per cell."""
    return 37 * 8 * nx * ny * nz
