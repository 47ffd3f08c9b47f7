"""Per-kernel timing of the granular, reference-shaped entry points: one
ht3d_<Kernel> per ParallelStencil @parallel kernel of
Dimensionless/kernels_HT3D.jl, Dimensional/kernels_HT3D_dimensional.jl,
tools/Macros.jl and tools/Weno5_Routines[_v2].jl, each called on its own the
way a driver loop calls the reference kernel.

  python -m hydrothermal3d_gb300.granular --n 255 --reps 5 [--md out.md] [--only REGEX]

Every kernel runs `reps` times between CUDA events on the context's stream
after two untimed calls.  At 255^3 one cell array of doubles is 133 MB, more
than the 129 MB L2, so each timed call streams its arrays from HBM.
Algorithmic bytes: each array the kernel reads is read once and each array
it writes is written once, counted over the cells the kernel touches (the
interior of a ghosted array that it updates in place).  Kernels that touch
only ghost faces (face BCs) are launch-bound; they are listed with their time
and their face bytes.  The dimensional BC kernels count one scan of the phase
array plus the ghost faces and the air and immersed rows they write.  Prints one JSON line per kernel and, with --md, writes
the table."""
import argparse
import json
import os
import re

import numpy as np
import torch

import hydrothermal3d_gb300 as ht
from hydrothermal3d_gb300 import api, v18


def _numel(shape):
    return int(np.prod(shape))


def shapes(n):
    return api._shapes(n, n, n)


def face_cells(n):
    """Cells on the six ghost faces of an (n+2)^3 array."""
    return 6 * (n + 2) ** 2


def kernels(ctx, n, seed=0):
    """(name, reference kernel, call, read shapes, written shapes) for every
    granular entry point; shapes are keys of shapes(n) or explicit cell
    counts (int)."""
    g = torch.Generator(device="cuda").manual_seed(seed)
    S = shapes(n)
    u = lambda key, lo=0.0, hi=1.0: api.zeros(*S[key]).uniform_(lo, hi, generator=g)
    h = 1.0 / n
    f = {}
    f["A"], f["P"] = u("ex"), u("ex")
    f["kx"], f["ky"], f["kz"] = u("fx", .5, 2), u("fy", .5, 2), u("fz", .5, 2)
    f["qx"], f["qy"], f["qz"] = u("fx", -1, 1), u("fy", -1, 1), u("fz", -1, 1)
    f["Ty"], f["Vx"], f["Vy"], f["Vz"] = u("fy"), u("fx", -1, 1), u("fy", -1, 1), u("fz", -1, 1)
    for name in ("R", "F", "F0", "G", "D", "rhoC", "Rt", "Rp", "Fc0", "Fcit", "c1", "c2", "c3", "c4", "c5", "Fold"):
        f[name] = u("c", .5, 1.5)
    f["kv"] = u("v", .5, 2)
    f["X3"] = u("xxx")
    # dimensional fields: the v18 box (crust, air ghost row, log-normal k), plus seeded fault/pluton/immersed cells
    b = v18.box(n, n, n, seed=2)
    p = b["params"]
    T, P, phc, phv, wN, kmul = (ht.from_numpy(b[k]) for k in ("T", "P", "phc", "phv", "wN", "kmul"))
    codes = torch.tensor([0.0, 0.0, 0.0, 2.0, 3.0], dtype=torch.float64, device="cuda")
    inner = phc[1:-1, 1:-1, 1:-1]
    inner.copy_(codes[torch.randint(0, codes.numel(), tuple(inner.shape), generator=g, device="cuda")])
    phc[1:-1, -2, 1:-1] = -1.0  # an immersed row under the air row
    f["Tc0"] = api.zeros(n, n, n).copy_(T[1:-1, 1:-1, 1:-1])
    f["Pc0"] = api.zeros(n, n, n).copy_(P[1:-1, 1:-1, 1:-1])
    kt = api.zeros(*S["v"])
    torch.cuda.synchronize()  # inputs were built on torch's stream
    bt, bv = [0, 0, 1, 1, 0, 0], [0, 0, 1.0, 0.0, 0, 0]
    F = f
    K = []
    add = lambda name, ref, call, reads, writes: K.append((name, ref, call, reads, writes))
    # ---------------------------------------------------------- dimensionless (Dimensionless/kernels_HT3D.jl)
    add("ComputeFlux", "ComputeFlux!", lambda: api.ComputeFlux(ctx, F["qx"], F["qy"], F["qz"], F["kx"], F["ky"], F["kz"],
                                                              F["A"], h, h, h),
        ["fx", "fy", "fz", "ex"], ["fx", "fy", "fz"])
    add("ResidualDiffusion", "ResidualDiffusion!",
        lambda: api.ResidualDiffusion(ctx, F["F"], F["R"], F["qx"], F["qy"], F["qz"], h, h, h),
        ["c", "fx", "fy", "fz"], ["c"])
    add("ResidualDiffusionTransient", "ResidualDiffusionTransient!",
        lambda: api.ResidualDiffusionTransient(ctx, F["F"], F["A"], F["R"], F["qx"], F["qy"], F["qz"], 2.0, h, h, h),
        ["c", "c", "fx", "fy", "fz"], ["c"])
    add("UpdateT", "UpdateT!",
        lambda: api.UpdateT(ctx, F["F"], F["A"], F["R"], F["qx"], F["qy"], F["qz"], 2.0, 1e-9, h, h, h),
        ["c", "c", "fx", "fy", "fz"], ["c", "c"])
    add("UpdateP", "UpdateP!", lambda: api.UpdateP(ctx, F["F0"], F["P"], F["F"], 0.99, 1e-9),
        ["c", "c", "c"], ["c", "c"])
    add("DYRELUpdate", "DYRELUpdate!", lambda: api.DYRELUpdate(ctx, F["F0"], F["P"], F["F"], 0.99, 0.5, 1e-9),
        ["c", "c", "c"], ["c", "c"])
    add("InitDarcy", "InitDarcy!", lambda: api.InitDarcy(ctx, F["Ty"], F["kx"], F["ky"], F["kz"], F["A"], F["kv"], 1.0),
        ["ex", "v"], ["fy", "fx", "fy", "fz"])
    add("InitThermal", "InitThermal!",
        lambda: api.InitThermal(ctx, F["Rt"], F["kx"], F["ky"], F["kz"], F["A"], F["kv"], 1.0),
        ["ex", "v"], ["c", "fx", "fy", "fz"])
    add("Compute_Rp", "Compute_Rp!", lambda: api.Compute_Rp(ctx, F["Rp"], F["ky"], F["Ty"], 100.0, n),
        ["fy", "fy"], ["c"])
    add("Init_vel", "Init_vel!",
        lambda: api.Init_vel(ctx, F["Vx"], F["Vy"], F["Vz"], F["kx"], F["ky"], F["kz"], F["P"], F["Ty"], 100.0, h, h, h),
        ["fx", "fy", "fz", "ex", "fy"], ["fx", "fy", "fz"])
    add("SetPressureBCs", "SetPressureBCs!", lambda: api.SetPressureBCs(ctx, F["P"], 0.0, 0.0),
        [face_cells(n)], [face_cells(n)])
    add("SetFaceBCs", "SetTemperatureBCs! (dimensionless)", lambda: api.SetFaceBCs(ctx, F["A"], bt, bv),
        [face_cells(n)], [face_cells(n)])
    add("KillNorthSouthFluxes", "KillNorthSouthFluxes!", lambda: api.KillNorthSouthFluxes(ctx, F["Ty"]),
        [], [2 * n * n])
    # ---------------------------------------------------------- DYREL support (Dimensional/kernels_HT3D_dimensional.jl)
    add("GershgorinPoisson", "GershgorinPoisson!",
        lambda: api.GershgorinPoisson(ctx, F["G"], F["D"], F["rhoC"], F["kx"], F["ky"], F["kz"], 1, 1.0, h, h, h),
        ["c", "fx", "fy", "fz"], ["c", "c"])
    add("GershgorinHydro", "GershgorinHydro!",
        lambda: api.GershgorinHydro(ctx, F["G"], F["rhoC"], F["kx"], F["ky"], F["kz"], 1, 1.0, h, h, h),
        ["c", "fx", "fy", "fz"], ["c"])
    add("SwapDYREL", "SwapDYREL!", lambda: api.SwapDYREL(ctx, F["c1"], F["c2"], F["A"], F["c3"]),
        ["c", "c"], ["c", "c"])
    add("RayleighQuotientNumerator", "RayleighQuotientNumerator!",
        lambda: api.RayleighQuotientNumerator(ctx, F["G"], F["Fc0"], F["Fcit"], F["F"], 1e-3),
        ["c", "c", "c"], ["c"])
    add("RayleighQuotientDenominator", "RayleighQuotientDenominator!",
        lambda: api.RayleighQuotientDenominator(ctx, F["G"], F["Fc0"], 1e-3), ["c"], ["c"])
    # ---------------------------------------------------------- reductions and copies (tools/Macros.jl)
    add("sum_g (ht3d_reduce)", "sum_g / mean_g", lambda: api.sum_g(ctx, F["R"]), ["c"], [])
    add("maximum_g (ht3d_reduce)", "maximum_g", lambda: api.maximum_abs_g(ctx, F["R"]), ["c"], [])
    add("Cpy_inn_to_all", "Cpy_inn_to_all!", lambda: api.Cpy_inn_to_all(ctx, F["c1"], F["A"]), ["c"], ["c"])
    add("Cpy_all_to_inn", "Cpy_all_to_inn!", lambda: api.Cpy_all_to_inn(ctx, F["A"], F["c1"]), ["c"], ["c"])
    add("ArrayEqualArray", "ArrayEqualArray!", lambda: api.ArrayEqualArray(ctx, F["c4"], F["c5"]), ["c"], ["c"])
    add("Multiply", "Multiply!", lambda: api.Multiply(ctx, F["c4"], F["c5"], F["R"]), ["c", "c"], ["c"])
    add("ResetA", "ResetA!", lambda: api.ResetA(ctx, F["c4"], F["c5"]), [], ["c", "c"])
    # ---------------------------------------------------------- WENO5 (tools/Weno5_Routines.jl, _v2.jl)
    add("VPlusMinus (x)", "VxPlusMinus!", lambda: api.VPlusMinus(ctx, F["c1"], F["c2"], F["Vx"], 0),
        ["fx"], ["c", "c"])
    add("Boundaries_Weno5 (x)", "Boundaries_x_Weno5!",
        lambda: api.Boundaries_Weno5(ctx, F["X3"], F["A"], 0, 1, 0.0, 1, 0.0), ["c"], ["c", 6 * n * n])
    add("Gradients_Weno5 (x, minus)", "Gradients_minus_x_Weno5!",
        lambda: api.Gradients_Weno5(ctx, F["c1"], F["c2"], F["c3"], F["c4"], F["c5"], F["X3"], 0, -1, n, n, n),
        ["c"], ["c"] * 5)
    add("dFdx_Weno5", "dFdx_Weno5!",
        lambda: api.dFdx_Weno5(ctx, F["D"], F["c1"], F["c2"], F["c3"], F["c4"], F["c5"]), ["c"] * 5, ["c"])
    add("Advect_v1", "Advect! (v1)",
        lambda: api.Advect_v1(ctx, F["Fold"], F["c1"], F["c2"], F["c3"], F["c4"], 1e-9), ["c"] * 5, ["c"])
    add("TimeAveraging_v1", "TimeAveraging! (v1)", lambda: api.TimeAveraging_v1(ctx, F["Fold"], F["c5"], 2),
        ["c", "c"], ["c"])
    add("Advect_v2 (x)", "Advect! (v2)",
        lambda: api.Advect_v2(ctx, F["A"], F["X3"], F["Vx"], 0, 1e-9, n, n, n), ["c", "c", "fx"], ["c"])
    add("TimeAveraging_v2", "TimeAveraging! (v2)", lambda: api.TimeAveraging_v2(ctx, F["A"], F["Fold"], 2),
        ["c", "c"], ["c"])
    # ---------------------------------------------------------- dimensional (Dimensional/kernels_HT3D_dimensional.jl)
    add("ComputeThermalConductivity", "ComputeThermalConductivity!",
        lambda: api.ComputeThermalConductivity(ctx, kt, T, phv, p.phi_i, p.sc_kt, p.sc_T), ["ex", "v"], ["v"])
    add("ComputeHydroConductivity", "ComputeHydroConductivity!",
        lambda: api.ComputeHydroConductivity(ctx, F["kv"], T, P, phv, p.ymin, p.dy, p.k_fact, p.delta, p.sc_sigma,
                                             p.sc_T, p.sc_L, p.sc_t, p.sc_eta, 1, kmul),
        ["ex", "ex", "v", "v"], ["v"])
    add("ComputeFluidDensity", "ComputeFluidDensity!",
        lambda: api.ComputeFluidDensity(ctx, F["kv"], T, P, phv, p.sc_sigma, p.sc_T, p.sc_rho), ["ex", "ex", "v"],
        ["v"])
    add("SmoothConductivityV2C", "SmoothConductivityV2C!", lambda: api.SmoothConductivityV2C(ctx, F["c1"], kt),
        ["v"], ["c"])
    add("SmoothConductivityC2V", "SmoothConductivityC2V!", lambda: api.SmoothConductivityC2V(ctx, kt, F["c1"]),
        ["c"], ["v"])
    add("InitConductivity", "InitConductivity!", lambda: api.InitConductivity(ctx, F["kx"], F["ky"], F["kz"], kt),
        ["v"], ["fx", "fy", "fz"])
    add("ComputeRhoCeffective", "ComputeRhoCeffective!",
        lambda: api.ComputeRhoCeffective(ctx, F["rhoC"], T, P, phc, p.phi_i, p.sc_T, p.sc_sigma, p.sc_C, p.sc_rho),
        ["c", "c", "c"], ["c"])
    add("ResidualTemperatureLinearised", "ResidualTemperatureLinearised!",
        lambda: api.ResidualTemperatureLinearised(ctx, F["F"], T, F["Tc0"], F["rhoC"], phc, F["R"], F["qx"], F["qy"],
                                                  F["qz"], 0.0, 1, 1.0 / p.dt, 1 / p.dx, 1 / p.dy, 1 / p.dz),
        ["c", "c", "c", "c", "c", "fx", "fy", "fz"], ["c"])
    add("SetTemperatureBCs (dimensional)", "SetTemperatureBCs!",
        lambda: api.SetTemperatureBCs(ctx, T, F["ky"], wN, phc, p.qyS, 1 / p.dy, 1.0, p.Tbot, p.Ttop),
        ["ex"], [face_cells(n) + 2 * n * n])
    add("SetPressureBCs (dimensional)", "SetPressureBCs! (dimensional)",
        lambda: api.SetPressureBCs_dim(ctx, P, wN, phc, p.Pbot, p.Ptop), ["ex"], [face_cells(n) + 2 * n * n])
    add("PhiRhof", "ϕρf!", lambda: api.PhiRhof(ctx, F["c1"], T, P, phc, p.phi_i, p.sc_rho, p.sc_T, p.sc_sigma),
        ["c", "c", "c"], ["c"])
    add("PhiRhofOld", "ϕρf_old!",
        lambda: api.PhiRhofOld(ctx, F["c2"], F["Tc0"], F["Pc0"], phc, p.phi_i, p.sc_rho, p.sc_T, p.sc_sigma),
        ["c", "c", "c"], ["c"])
    add("PhiDrhodP", "ϕdρdP!", lambda: api.PhiDrhodP(ctx, F["c3"], T, P, phc, p.phi_i, p.sc_rho, p.sc_T, p.sc_sigma),
        ["c", "c", "c"], ["c"])
    add("ComputeDarcyFlux", "ComputeDarcyFlux!",
        lambda: api.ComputeDarcyFlux(ctx, F["qx"], F["qy"], F["qz"], F["kv"], F["kx"], F["ky"], F["kz"], P, p.g,
                                     1 / p.dx, 1 / p.dy, 1 / p.dz),
        ["v", "fx", "fy", "fz", "ex"], ["fx", "fy", "fz"])
    add("ResidualFluidPressure", "ResidualFluidPressure!",
        lambda: api.ResidualFluidPressure(ctx, F["F"], phc, F["c1"], F["c2"], F["R"], F["qx"], F["qy"], F["qz"], 1,
                                          1.0 / p.dt, 1 / p.dx, 1 / p.dy, 1 / p.dz),
        ["c", "c", "c", "c", "fx", "fy", "fz"], ["c"])
    add("Init_vel_dim", "Init_vel! (dimensional)",
        lambda: api.Init_vel_dim(ctx, F["Vx"], F["Vy"], F["Vz"], F["qx"], F["qy"], F["qz"], F["kv"]),
        ["fx", "fy", "fz", "v"], ["fx", "fy", "fz"])
    return K, S


def nbytes(keys, S):
    return 8 * sum(k if isinstance(k, int) else _numel(S[k]) for k in keys)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=255)
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--md", default=None, help="write the table as markdown to this path")
    ap.add_argument("--only", default=None, help="run only the entry points whose name matches this regex")
    a = ap.parse_args()
    stream = torch.cuda.Stream()
    ctx = ht.Context(device=0, stream=stream.cuda_stream, sync=False)
    try:
        with open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                               "MEASURED_PEAKS.json")) as fh:
            peak, peak_src = float(json.load(fh)["hbm_gbs"]), "of measured"
    except (OSError, KeyError, ValueError):
        peak, peak_src = 6800.0, "of fallback"
    K, S = kernels(ctx, a.n)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    rows = []
    if a.only:
        K = [kk for kk in K if re.search(a.only, kk[0])]
    for name, ref, call, reads, writes in K:
        call()
        call()
        ctx.synchronize()
        e0.record(stream)
        for _ in range(a.reps):
            call()
        e1.record(stream)
        torch.cuda.synchronize()
        us = e0.elapsed_time(e1) / a.reps * 1e3
        alg = nbytes(reads, S) + nbytes(writes, S)
        row = {"kernel": name, "reference": ref, "us": round(us, 2), "alg_MB": round(alg / 1e6, 1),
               "GBs": round(alg / us / 1e3, 1), "frac": round(alg / us / 1e3 / peak, 3), "n": a.n}
        rows.append(row)
        print(json.dumps(row), flush=True)
    if a.md:
        with open(a.md, "w") as fh:
            fh.write(f"| ht3d entry point | reference kernel | us / call | algorithmic MB | GB/s | frac ({peak_src} "
                     f"{peak:.0f} GB/s) |\n|---|---|---|---|---|---|\n")
            for r in rows:
                fh.write(f"| `{r['kernel']}` | `{r['reference']}` | {r['us']:.1f} | {r['alg_MB']:.1f} | {r['GBs']:.0f} "
                         f"| {r['frac']:.2f} |\n")


if __name__ == "__main__":
    main()
