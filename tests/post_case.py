"""Shared inputs of the output-diagnostic tests: a ghosted grid with every
phase code the dimensional model uses (-1 immersed, 0 crust, 1 air, 2 fault,
3 pluton), dimensional scales of the v18 driver's order of magnitude, and the
oracle's output of every diagnostic."""
import numpy as np

PARAMS = dict(phi0=0.01, scale_T=600.0, scale_sigma=1e8, scale_V=1e-9, scale_L=1e3, k_fact=100.0, ymin=-30.0,
              dy=0.25, delta=2.0)
SENTINEL = -7.25  # initial value of every output: shows which cells a kernel leaves untouched


def case(nx=13, ny=11, nz=6, seed=5):
    rng = np.random.default_rng(seed)
    ex = (nx + 2, ny + 2, nz + 2)
    phc = np.asfortranarray(rng.choice([-1.0, 0.0, 1.0, 2.0, 3.0], size=ex, p=[0.1, 0.4, 0.2, 0.2, 0.1]))
    return dict(
        n=(nx, ny, nz),
        phc=phc,
        T=np.asfortranarray(rng.uniform(0.5, 1.5, ex)),
        P=np.asfortranarray(rng.uniform(1e-3, 3.0, ex)),
        Vx=np.asfortranarray(rng.uniform(-1, 1, (nx + 1, ny, nz))),
        Vy=np.asfortranarray(rng.uniform(-1, 1, (nx, ny + 1, nz))),
        Vz=np.asfortranarray(rng.uniform(-1, 1, (nx, ny, nz + 1))),
    )


def out(n):
    return np.full(n, SENTINEL, order="F")


def oracle_fields(orc, c):
    """Every diagnostic from the oracle's per-kernel restatements, keyed by the
    ht3d_post_fields names."""
    p, n = PARAMS, c["n"]
    r = {k: out(n) for k in ("phase", "pressure", "temperature", "vx", "vy", "vz", "k_thermal", "heat_capacity",
                             "permeability", "density", "viscosity", "peclet")}
    orc.call("Phase", r["phase"], c["phc"], *n)
    orc.call("Pressure", r["pressure"], c["P"], c["phc"], p["scale_sigma"], *n)
    orc.call("Temperature", r["temperature"], c["T"], c["phc"], p["scale_T"], *n)
    orc.call("Velocity", r["vx"], r["vy"], r["vz"], c["Vx"], c["Vy"], c["Vz"], c["phc"], p["scale_V"], *n)
    orc.call("EffectiveThermalConductivity", r["k_thermal"], c["T"], p["phi0"], c["phc"], p["scale_T"], *n)
    orc.call("EffectiveHeatCapacity", r["heat_capacity"], c["T"], c["P"], c["phc"], p["phi0"], p["scale_T"],
             p["scale_sigma"], 1.0, 1.0, *n)
    orc.call("Permeability", r["permeability"], p["k_fact"], p["ymin"], p["dy"], c["phc"], p["delta"], p["scale_L"], *n)
    orc.call("FluidDensity", r["density"], c["T"], c["P"], c["phc"], p["scale_T"], p["scale_sigma"], *n)
    orc.call("Viscosity", r["viscosity"], c["T"], c["phc"], p["scale_T"], *n)
    orc.call("Peclet", r["peclet"], c["T"], c["P"], c["Vx"], c["Vy"], c["Vz"], c["phc"], p["phi0"], p["scale_T"],
             p["scale_sigma"], p["scale_V"], p["scale_L"], *n)
    return r
