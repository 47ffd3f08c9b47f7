#!/usr/bin/env python
"""Benchmark of the HydroThermal3D pseudo-transient hot path on GB300.

Workload: the dimensionless Horton-Rogers-Lapwood convection problem
(Ra = 1000, unit cube, T linear 1 -> 0 plus a seeded 1e-3 perturbation,
DYREL tolerance 1e-8, WENO5 advection, adaptive dt) at 255^3 cells.
A step is one full time step: thermal DYREL solve, Darcy DYREL solve,
Darcy velocity, WENO5 advection, dt update.

Metric: T_eff (GB/s) = algorithmic bytes / wall time, where a DYREL
pseudo-iteration counts 9*N*s bytes and a WENO5 advection 21*N*s bytes
(s = storage width: 4 B for the mixed form, 8 B for FP64).  `value` is the
mixed-precision form; the FP64 form, time-steps/s and the mixed-vs-FP64 error
are reported beside it.

  python bench.py [--steps K] [--warmup W] [--n 255] [--impl reference]
Under torchrun with N > 1 every rank runs an independent replica on its own
GPU (the path has no exchange step); value = all ranks' bytes / max time.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "T_eff GB/s & time-steps/s at 255^3: FP32-mixed vs FP64 GPU at 1e-6 rel err in T"
UNIT = "GB/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=255)
    ap.add_argument("--nitout", type=int, default=1000)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--ens-members", type=int, default=64)
    ap.add_argument("--ens-steps", type=int, default=20)
    ap.add_argument("--skip-ensemble", action="store_true")
    ap.add_argument("--mixed-refresh", type=int, default=0,
                    help="FP64 refresh cadence of the mixed form in inner iterations (0 = library default)")
    ap.add_argument("--temporal", type=int, default=-1,
                    help="two inner iterations per pass of the mixed form (HT3D_TUNE_TEMPORAL; -1 = library default)")
    ap.add_argument("--nu-steps", type=int, default=60,
                    help="time steps of the 63^3 Nusselt time series, FP64 vs mixed (0 = skip)")
    ap.add_argument("--post-n", type=int, default=255, help="cells per axis of the output-diagnostics pass (0 = skip)")
    ap.add_argument("--sweep-n", type=int, default=511, help="cells per axis of the standalone WENO5 sweep (0 = skip)")
    ap.add_argument("--c63-steps", type=int, default=10,
                    help="time steps of the 63^3 HRL case (config 1): oracle on the host cores and GPU forms "
                         "(0 = skip)")
    ap.add_argument("--growth-steps", type=int, default=6,
                    help="steps of the 127^3 error-growth comparison (mixed and a 1e-8-perturbed FP64 run "
                         "against FP64; 0 = skip)")
    ap.add_argument("--v18-steps", type=int, default=2,
                    help="time steps of the 127^3 dimensional (v18) box, plain FP64 (0 = skip)")
    ap.add_argument("--v18-nitmax", type=int, default=100000,
                    help="DYREL iteration cap of the dimensional box (the reference's 1e4 stops the 127^3 Darcy "
                         "solves before the 1e-10 tolerance)")
    ap.add_argument("--c127-steps", type=int, default=0,
                    help="first time steps of the 127^3 dimensional box on the oracle (host cores) against the "
                         "GPU FP64 form: T, P, V errors (0 = skip; minutes of host time per step)")
    ap.add_argument("--fault-steps", type=int, default=0,
                    help="time steps of the 511^3 fault-slab HRL case (mixed form; 0 = skip)")
    ap.add_argument("--c3-steps", type=int, default=0,
                    help="time steps of the 255^3 mixed-vs-FP64 accuracy study (100 as the workload states it; "
                         "0 = skip)")
    ap.add_argument("--c3-n", type=int, default=255, help="cells per axis of the accuracy study")
    ap.add_argument("--c3-cadence-control", type=int, default=500,
                    help="check cadence of the accuracy study's second FP64 control (0 = no such control)")
    ap.add_argument("--c3-out", default="",
                    help="also write the accuracy study's record (one JSON object) to this file")
    return ap.parse_args()


def workload_config(a, extra=None):
    c = {"workload": f"HRL porous convection {a.n}^3 (Ra=1000, DYREL tol 1e-8, nitout {a.nitout}, WENO5 v1, adaptive dt)",
         "cells": a.n ** 3, "Ra": 1000.0, "dyrel_tol": 1e-8, "nitout": a.nitout,
         "l2_policy": "inputs larger than L2 (each 255^3 FP64 field is 133 MB > 129 MB L2)",
         "parallelism": f"replicas x{a.gpus}"}
    if getattr(a, "mixed_refresh", 0):
        c["mixed_refresh"] = a.mixed_refresh
    if getattr(a, "temporal", -1) >= 0:
        c["temporal"] = a.temporal
    if extra:
        c.update(extra)
    return c


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """Samples nvidia-smi SM clocks and throttle reasons during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 6:
                continue
            try:
                sm.append(float(f[0]))
                mx = max(mx, float(f[1]))
            except ValueError:
                continue
            for nm, v in zip(names, f[2:6]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ distributed
def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def reduce_max_sum(ws, t, units):
    from hydrothermal3d_gb300.replicas import max_time_sum_units
    return max_time_sum_units(t, units) if ws > 1 else (t, units)


# ------------------------------------------------------------------ CPU baseline
def cpu_sample(n, seconds, threads=None):
    """Time the oracle (unfused FP64, OpenMP over z) on a bounded sample of the
    workload: DYREL pseudo-iterations of both solves plus WENO5 advections at
    the same grid.  Returns (T_eff GB/s, cores, description)."""
    import oracle
    from hydrothermal3d_gb300 import hrl, abi
    if threads:
        oracle.set_threads(threads)
    cores = oracle.num_threads()
    T, P, ktv, kfv = hrl.initial_fields(n, n, n, seed=1)
    nx = ny = nz = n
    d = 1.0 / n
    R = np.asfortranarray(-T[1:-1, 1:-1, 1:-1] / (d * d / 6.1))
    k = [np.ones(s, order="F") for s in ((nx + 1, ny, nz), (nx, ny + 1, nz), (nx, ny, nz + 1))]
    F, F0 = oracle.zeros(nx, ny, nz), oracle.zeros(nx, ny, nz)
    V = [np.asfortranarray(np.random.default_rng(2).uniform(-1, 1, s)) for s in ((nx + 1, ny, nz), (nx, ny + 1, nz), (nx, ny, nz + 1))]
    prm = abi.DyrelParams.reference(nitout=1000)
    tb = oracle.int6(0, 0, 1, 1, 0, 0)
    tv = oracle.dbl6(0, 0, 1, 0, 0, 0)
    iters, adv, t_tot = 0, 0, 0.0
    chunk = 10
    while t_tot < seconds or iters == 0:
        t0 = time.perf_counter()
        oracle.dyrel_solve_dimless(T, R, *k, 6.1 / (d * d), d, d, d, [0, 0, 1, 1, 0, 0], [0, 0, 1, 0, 0, 0], prm, F, F0,
                                   n_iter_fixed=chunk)
        oracle.dyrel_solve_dimless(P, R, *k, 0.0, d, d, d, [0] * 6, [0.0] * 6, prm, F, F0, n_iter_fixed=chunk)
        oracle.call("AdvectWithWeno5_v1", T, *V, 1e-4, float(n), float(n), float(n), tb, tv, nx, ny, nz)
        t_tot += time.perf_counter() - t0
        iters += 2 * chunk
        adv += 1
    nbytes = iters * hrl.bytes_per_iteration(n, n, n, 8) + adv * hrl.bytes_per_advection(n, n, n, 8)
    desc = (f"oracle FP64 at {n}^3: {iters} DYREL pseudo-iterations (thermal+Darcy, incl. per-solve Gershgorin set-up)"
            f" + {adv} WENO5 advections in {t_tot:.1f} s")
    cell_updates = iters * n ** 3 / t_tot  # pseudo-iteration cell updates per second (advection time included)
    return nbytes / t_tot / 1e9, cores, desc, t_tot, cell_updates


def oracle_c63(steps, threads=None):
    """Config 1: the oracle (C++ FP64, OpenMP) runs `steps` full HRL time steps
    at 63^3 from the seeded initial condition on the host cores.  Returns the
    timing summary and the final (T, P) for the GPU parity check."""
    import oracle
    from hydrothermal3d_gb300 import hrl
    if threads:
        oracle.set_threads(threads)
    n = 63
    T, P, ktv, kfv = hrl.initial_fields(n, n, n, seed=1)
    p = hrl.params(n, n, n)
    V = [np.zeros(s, order="F") for s in ((n + 1, n, n), (n, n + 1, n), (n, n, n + 1))]
    iters, nbytes = [], 0
    t0 = time.perf_counter()
    for _ in range(steps):
        st, a_, b_ = oracle.step_hrl(T, P, ktv, kfv, *V, p)
        iters.append([a_.iters, b_.iters])
        nbytes += (a_.iters + b_.iters) * hrl.bytes_per_iteration(n, n, n, 8) + hrl.bytes_per_advection(n, n, n, 8)
    t = time.perf_counter() - t0
    res = {"n": n, "steps": steps, "seconds": t, "time_steps_per_s": steps / t, "T_eff_GBs": nbytes / t / 1e9,
           "cores": oracle.num_threads(), "pseudo_iterations_per_step": iters,
           "impl": "oracle (C++ FP64, unfused kernels, OpenMP)"}
    return res, T, P


def c63_bench(ctx, stream, steps):
    """Config 1 on the GPU (FP64 and mixed forms, same 63^3 workload and steps
    as the oracle run beside it); the FP64 form's final fields are compared
    with the oracle's."""
    import torch
    import hydrothermal3d_gb300 as ht
    from hydrothermal3d_gb300 import api, abi, hrl
    cpu, To, Po = oracle_c63(steps, threads=os.cpu_count())
    n = 63
    T0, P0, ktv, kfv = hrl.initial_fields(n, n, n, seed=1)
    ktd, kfd = ht.from_numpy(ktv), ht.from_numpy(kfv)
    V = [ht.zeros(n + 1, n, n), ht.zeros(n, n + 1, n), ht.zeros(n, n, n + 1)]
    res = {"cpu_oracle": cpu}
    inner = (slice(1, -1),) * 3
    for name, prec, s in (("gpu_fp64", abi.FP64, 8), ("gpu_mixed", abi.MIXED, 4)):
        Td, Pd = ht.from_numpy(T0), ht.from_numpy(P0)
        p = hrl.params(n, n, n)
        nbytes = 0
        with torch.cuda.stream(stream):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for _ in range(steps):
                gt, gd = api.step_hrl(ctx, Td, Pd, ktd, kfd, *V, p, prec)
                nbytes += (gt.iters + gd.iters) * hrl.bytes_per_iteration(n, n, n, s) + \
                    hrl.bytes_per_advection(n, n, n, s)
            torch.cuda.synchronize()
            t = time.perf_counter() - t0
        Tg = ht.to_numpy(Td)
        Pg = ht.to_numpy(Pd)
        Pg_, Po_ = Pg[inner] - Pg[inner].mean(), Po[inner] - Po[inner].mean()
        res[name] = {"time_steps_per_s": steps / t, "T_eff_GBs": nbytes / t / 1e9, "seconds": t,
                     "T_rel_err_vs_oracle": float(np.abs(Tg[inner] - To[inner]).max() / np.abs(To[inner]).max()),
                     "P_rel_err_vs_oracle_mean_removed": float(np.abs(Pg_ - Po_).max() / np.abs(Po_).max()),
                     "T_bitwise_equal_to_oracle": bool(np.array_equal(Tg[inner], To[inner]))}
    res["note"] = ("63^3 fields fit in L2 (each FP64 field ~2 MB), so GPU T_eff here is not an HBM figure; "
                   "the accumulated mixed error includes the growth of perturbations through the convective "
                   "instability over the steps")
    return res


def run_reference(a):
    ws, rank, _ = dist_setup()
    if rank != 0:
        return
    cores = os.cpu_count()
    vals = []
    cups = []
    for s in range(a.warmup + a.steps):
        v, cores, desc, _, cu = cpu_sample(a.n, max(2.0, a.cpu_seconds / 4), threads=os.cpu_count())
        if s >= a.warmup:
            vals.append(v)
            cups.append(cu)
    value = float(np.mean(vals))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": a.gpus, "steps": a.steps,
            "warmup": a.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded HRL initial condition)",
            "config": workload_config(a, {"reference_impl": "CPU oracle port (reference is Julia; not runnable here)"}),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": desc},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "cell_updates_per_s": float(np.mean(cups)),
            "work_note": ("T_eff counts 8 B per field value here and 4 B in the mixed GPU form; cell_updates_per_s "
                          "(DYREL pseudo-iterations x cells per second, advection time included) compares the arms "
                          "at equal work. Each step is a bounded sample of the workload, not a full time step: one "
                          "255^3 FP64 time step takes minutes on the host cores")}
    if a.c63_steps:
        line["config_63"] = oracle_c63(a.c63_steps, threads=os.cpu_count())[0]
    print(json.dumps(line))


# ------------------------------------------------------------------ GPU arm
def run_ours(a):
    import torch
    import hydrothermal3d_gb300 as ht
    from hydrothermal3d_gb300 import api, abi, hrl

    ws, rank, local = dist_setup()
    dev = local if torch.cuda.is_available() else 0
    torch.cuda.set_device(dev)
    stream = torch.cuda.Stream()
    ctx = ht.Context(device=dev, stream=stream.cuda_stream)
    if a.mixed_refresh:
        ctx.set_tuning(abi.TUNE_MIXED_REFRESH, a.mixed_refresh)
    if a.temporal >= 0:
        ctx.set_tuning(abi.TUNE_TEMPORAL, a.temporal)
    n = a.n
    N = n ** 3
    T0, P0, ktv, kfv = hrl.initial_fields(n, n, n, seed=1)
    ktd, kfd = ht.from_numpy(ktv), ht.from_numpy(kfv)
    Vd = [ht.zeros(n + 1, n, n), ht.zeros(n, n + 1, n), ht.zeros(n, n, n + 1)]
    torch.cuda.synchronize()

    def run_form(prec, steps, warmup, sampler=None):
        Td, Pd = ht.from_numpy(T0), ht.from_numpy(P0)
        p = hrl.params(n, n, n, nitout=a.nitout)
        s = 8 if prec == abi.FP64 else 4
        with torch.cuda.stream(stream):
            for _ in range(warmup):
                api.step_hrl(ctx, Td, Pd, ktd, kfd, *Vd, p, prec)
            torch.cuda.synchronize()
            barrier(ws)
            # the mixed solver times its FP32 inner-iteration runs on the ctx
            # stream during the timed steps (the roofline's kernel duration)
            ctx.set_tuning(abi.TUNE_TIME_INNER, 1 if prec == abi.MIXED else 0)
            ctx.inner_timing(reset=True)
            l0 = ctx.launches
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            iters, nbytes = [], 0
            cm = sampler if sampler is not None else _Null()
            with cm:
                e0.record(stream)
                for _ in range(steps):
                    gt, gd = api.step_hrl(ctx, Td, Pd, ktd, kfd, *Vd, p, prec)
                    iters.append((gt.iters, gd.iters))
                    nbytes += (gt.iters + gd.iters) * hrl.bytes_per_iteration(n, n, n, s) + hrl.bytes_per_advection(n, n, n, s)
                e1.record(stream)
                torch.cuda.synchronize()
            barrier(ws)
            ms = e0.elapsed_time(e1)
            inner = ctx.inner_timing(reset=True)
            ctx.set_tuning(abi.TUNE_TIME_INNER, 0)
        return dict(ms=ms, bytes=nbytes, iters=iters, launches=ctx.launches - l0, T=Td, P=Pd, params=p, inner=inner)

    sampler = ClockSampler(dev)
    mixed = run_form(abi.MIXED, a.steps, a.warmup, sampler)
    # end to end through the public API with host buffers (mixed form), right
    # after the device-timed steps of the same workload and before the FP64
    # arm (each step computes V before reading it: the runs are independent)
    e2e_res = e2e(ctx, stream, a, ktd, kfd, Vd)
    fp64 = None if a.skip_fp64 else run_form(abi.FP64, a.steps, a.warmup)
    t_mixed, b_mixed = reduce_max_sum(ws, mixed["ms"] / 1e3, mixed["bytes"])
    value = b_mixed / t_mixed / 1e9
    steps_per_s = a.steps * ws / t_mixed

    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": a.steps, "warmup": a.warmup,
           "ms_per_step": mixed["ms"] / a.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32+f64 (mixed)", "data": "synthetic (seeded HRL initial condition)",
           "config": workload_config(a), "time_steps_per_s": steps_per_s,
           "cell_updates_per_s": sum(x + y for x, y in mixed["iters"]) * N * ws / t_mixed,
           "pseudo_iterations_per_step": [list(x) for x in mixed["iters"]], "gpu_launches": mixed["launches"]}
    if fp64 is not None:
        t64, b64 = reduce_max_sum(ws, fp64["ms"] / 1e3, fp64["bytes"])
        out["fp64"] = {"T_eff_GBs": b64 / t64 / 1e9, "time_steps_per_s": a.steps * ws / t64,
                       "cell_updates_per_s": sum(x + y for x, y in fp64["iters"]) * N * ws / t64,
                       "ms_per_step": fp64["ms"] / a.steps,
                       "pseudo_iterations_per_step": [list(x) for x in fp64["iters"]]}
        out["mixed_vs_fp64_time_steps_speedup"] = steps_per_s / out["fp64"]["time_steps_per_s"]
        inner = (slice(1, -1),) * 3
        Tm, T6 = mixed["T"][inner], fp64["T"][inner]
        Pm, P6 = mixed["P"][inner], fp64["P"][inner]
        Pm, P6 = Pm - Pm.mean(), P6 - P6.mean()
        out["mixed_error_vs_fp64_gpu"] = {
            "accumulated_T_rel_maxnorm": float((Tm - T6).abs().max() / T6.abs().max()),
            "accumulated_P_rel_maxnorm_mean_removed": float((Pm - P6).abs().max() / P6.abs().max()),
            "after_steps": a.warmup + a.steps,
            "note": "accumulated values include the growth of any perturbation through the convective instability"}
        out["mixed_error_vs_fp64_gpu"].update(one_step_error(ctx, stream, a, fp64, ktd, kfd, Vd))
    out["clocks"] = sampler.summary()

    # --- roofline of the dominant kernel: the FP32 inner DYREL iteration of
    # the mixed form, timed live inside the timed steps above
    out["roofline"] = roofline(ctx, stream, n, mixed["inner"], mixed["ms"], pairs=a.temporal != 0)

    out["e2e"] = e2e_res

    # --- secondary metric: batched ensemble vs the same members one by one
    if not a.skip_ensemble:
        out["ensemble"] = ensemble_bench(ctx, stream, a)
    # --- standalone WENO5 sweep on the large grid
    if a.sweep_n:
        out["weno_sweep"] = sweep_bench(ctx, stream, a.sweep_n)
    if a.fault_steps:
        out["fault_slab_511"] = fault_bench(ctx, stream, a)
    if a.v18_steps:
        out["dimensional_127"] = v18_bench(ctx, stream, a.v18_steps, nitmax=a.v18_nitmax)
    if a.c127_steps and rank == 0:
        out["config_127"] = c127_bench(ctx, stream, a.c127_steps, nitmax=a.v18_nitmax)
    if a.growth_steps:
        out["error_growth_127"] = growth_bench(ctx, stream, a.growth_steps)
    if a.c63_steps and rank == 0:
        out["config_63"] = c63_bench(ctx, stream, a.c63_steps)
    if a.post_n:
        out["diagnostics"] = post_bench(ctx, stream, a.post_n)
    if a.nu_steps and rank == 0:
        out["nusselt_63"] = nusselt_bench(ctx, stream, a.nu_steps)
    if a.c3_steps and rank == 0:
        out["accuracy_255"] = accuracy_bench(ctx, stream, a.c3_steps, a.c3_n, a.c3_cadence_control, a.c3_out)

    if rank == 0:
        v, cores, desc, _, cu = cpu_sample(n, a.cpu_seconds, threads=os.cpu_count())
        out["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": desc,
                               "cell_updates_per_s": cu}
    if rank == 0:
        print(json.dumps(out))
    ctx.close()


def one_step_error(ctx, stream, a, fp64, ktd, kfd, Vd):
    """Error of one mixed-precision step against one FP64 step taken from the
    same (FP64) state: the error the mixed form adds per time step."""
    import torch
    import hydrothermal3d_gb300 as ht
    from hydrothermal3d_gb300 import api, abi, hrl
    n = a.n
    res = {}
    outs = {}
    for name, prec in (("fp64", abi.FP64), ("mixed", abi.MIXED)):
        Td, Pd = fp64["T"].clone(), fp64["P"].clone()
        Tc, Pc = ht.zeros(n + 2, n + 2, n + 2), ht.zeros(n + 2, n + 2, n + 2)
        Tc.copy_(Td)
        Pc.copy_(Pd)
        p = fp64["params"]
        q = hrl.params(n, n, n, nitout=a.nitout)
        q.dt = p.dt
        with torch.cuda.stream(stream):
            api.step_hrl(ctx, Tc, Pc, ktd, kfd, *Vd, q, prec)
        torch.cuda.synchronize()
        outs[name] = (Tc, Pc)
    inner = (slice(1, -1),) * 3
    T6, Tm = outs["fp64"][0][inner], outs["mixed"][0][inner]
    P6, Pm = outs["fp64"][1][inner], outs["mixed"][1][inner]
    P6, Pm = P6 - P6.mean(), Pm - Pm.mean()
    res["one_step_T_rel_maxnorm"] = float((Tm - T6).abs().max() / T6.abs().max())
    res["one_step_P_rel_maxnorm_mean_removed"] = float((Pm - P6).abs().max() / P6.abs().max())
    return res


class _Null:
    def __enter__(self):
        return self

    def __exit__(self, *e):
        return False


def roofline(ctx, stream, n, inner, step_ms, iters=20, pairs=True):
    import torch
    import hydrothermal3d_gb300 as ht
    from hydrothermal3d_gb300 import abi, hrl
    inner_ms, inner_iters = inner
    t = inner_ms / 1e3 / max(1, inner_iters)  # per pseudo-iteration
    alg = hrl.bytes_per_iteration(n, n, n, 4)
    peak = measured_peak()
    achieved = alg / t / 1e9
    traffic = profile_traffic("mixed_pair_f32" if pairs else "mixed_inner_f32")
    if pairs:
        kernel = ("k_mixed_inner2 (two FP32 pseudo-iterations of the mixed form per pass through memory, TMA-staged "
                  "planes, padded float4 layout)")
        note = ("two iterations per pass: per iteration the kernel reads the six streamed fields and writes one "
                "correction field once for every two iterations, so the algorithmic 9 fields per iteration exceed "
                "the DRAM bytes about 2.2-fold and achieved exceeds the copy peak; dram_frac is the measured DRAM "
                "bytes per iteration over the same time")
    else:
        kernel = "k_mixed_inner (FP32 pseudo-iteration of the mixed form, padded float4 layout)"
        note = ("the kernel streams 7 of the 9 algorithmic fields (the Jacobi diagonal is recomputed, the DYREL "
                "momentum is implied by the previous correction); dram_frac is the measured DRAM bytes per "
                "iteration over the same time")
    res = {"kernel": kernel, "bound": "hbm",
           "achieved": achieved, "peak": peak[0], "unit": "GB/s", "frac": achieved / peak[0], "peak_source": peak[1],
           "traffic": traffic, "traffic_unit": "DRAM bytes per pseudo-iteration",
           "dram_frac": (traffic / t / 1e9 / peak[0]) if traffic else None,
           "us_per_iteration": t * 1e6, "alg_bytes_per_iteration": alg, "iterations_timed": inner_iters,
           "share_of_timed_region": inner_ms / step_ms if step_ms else None,
           "timing": "CUDA events on the ctx stream around every run of consecutive inner launches inside the "
                     "timed steps (HT3D_TUNE_TIME_INNER)",
           "note": note}
    X64c = ht.zeros(n + 2, n + 2, n + 2).uniform_(0, 1)
    R64c = ht.zeros(n, n, n).uniform_(-1, 1)
    k64c = [ht.ones(n + 1, n, n), ht.ones(n, n + 1, n), ht.ones(n, n, n + 1)]
    iPCc = ht.ones(n, n, n) * (6.0 * n * n)
    F0c = ht.zeros(n, n, n)
    bt, bv = abi.int6(0, 0, 1, 1, 0, 0), abi.dbl6(0, 0, 1, 0, 0, 0)
    d = 1.0 / n
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    # FP64 form's kernel for comparison (FP64-ALU bound on GB300)
    a64 = lambda m: (X64c.data_ptr(), R64c.data_ptr(), k64c[0].data_ptr(), k64c[1].data_ptr(), k64c[2].data_ptr(),
                     iPCc.data_ptr(), F0c.data_ptr(), 0.0, d, d, d, bt, bv, 0.99, 0.05, 0.01, m, n, n, n)
    torch.cuda.synchronize()
    ctx.call("ht3d_dyrel_iterate", *a64(2))
    ctx.synchronize()
    e0.record(stream)
    ctx.call("ht3d_dyrel_iterate", *a64(iters))
    e1.record(stream)
    torch.cuda.synchronize()
    t64 = e0.elapsed_time(e1) / 1e3 / iters
    alg64 = hrl.bytes_per_iteration(n, n, n, 8)
    res["fp64_kernel"] = {"kernel": "k_dyrel_iter<double,PLAIN>", "us_per_launch": t64 * 1e6,
                          "achieved_GBs": alg64 / t64 / 1e9, "frac_hbm": alg64 / t64 / 1e9 / peak[0],
                          "fp64_alu_nominal_tflops": 1.25}
    return res


def e2e(ctx, stream, a, ktd, kfd, Vd):
    import torch
    import hydrothermal3d_gb300 as ht
    from hydrothermal3d_gb300 import api, abi, hrl
    n = a.n
    T0, P0, _, _ = hrl.initial_fields(n, n, n, seed=1)
    hT = torch.from_numpy(np.ascontiguousarray(T0.transpose(2, 1, 0))).pin_memory()
    hP = torch.from_numpy(np.ascontiguousarray(P0.transpose(2, 1, 0))).pin_memory()
    Td, Pd = ht.zeros(n + 2, n + 2, n + 2), ht.zeros(n + 2, n + 2, n + 2)
    p = hrl.params(n, n, n, nitout=a.nitout)
    nbytes = 0
    with torch.cuda.stream(stream):
        for w in range(2):  # warm-up of the copy path
            Td.permute(2, 1, 0).copy_(hT, non_blocking=True)
            hT.copy_(Td.permute(2, 1, 0), non_blocking=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(a.steps):
            Td.permute(2, 1, 0).copy_(hT, non_blocking=True)
            Pd.permute(2, 1, 0).copy_(hP, non_blocking=True)
            gt, gd = api.step_hrl(ctx, Td, Pd, ktd, kfd, *Vd, p, abi.MIXED)
            hT.copy_(Td.permute(2, 1, 0), non_blocking=True)
            hP.copy_(Pd.permute(2, 1, 0), non_blocking=True)
            stream.synchronize()
            nbytes += (gt.iters + gd.iters) * hrl.bytes_per_iteration(n, n, n, 4) + hrl.bytes_per_advection(n, n, n, 4)
        t = time.perf_counter() - t0
    per = 2 * (n + 2) ** 3 * 8
    return {"value": nbytes / t / 1e9, "unit": UNIT, "h2d_bytes_per_step": per, "d2h_bytes_per_step": per,
            "time_steps_per_s": a.steps / t, "note": "host-timed; pinned host T,P copied in and out every step"}


def ensemble_bench(ctx, stream, a):
    """Ensemble workload: members with n ~ U{31..95} per axis, Ra ~ logU[100, 5000]
    and independent log-normal permeability (seed 4), mixed form, ens-steps
    steps.  Batched arm: ht3d_ensemble_step; sequential arm: ht3d_step_hrl on
    each member in turn.  Both start from the same state and do the same
    work (bit-identical results); metric = cell updates (cells x DYREL
    pseudo-iterations) per second."""
    import torch
    import hydrothermal3d_gb300 as ht
    from hydrothermal3d_gb300 import api, abi, hrl
    base = hrl.ensemble(n_members=a.ens_members, seed=4)

    def make():
        mem = []
        for T, P, ktv, kfv, p in base:
            nx, ny, nz = (s - 2 for s in T.shape)
            mem.append(api.Member(ht.from_numpy(T), ht.from_numpy(P), ht.from_numpy(ktv), ht.from_numpy(kfv),
                                  ht.zeros(nx + 1, ny, nz), ht.zeros(nx, ny + 1, nz), ht.zeros(nx, ny, nz + 1),
                                  abi.HrlParams.from_buffer_copy(p)))
        return mem

    def reset(mem):
        for m, (T, P, _, _, p) in zip(mem, base):
            m.Tc_ex.copy_(ht.from_numpy(T))
            m.Pc_ex.copy_(ht.from_numpy(P))
            m.params = abi.HrlParams.from_buffer_copy(p)

    def step_batched(mem):
        api.ensemble_step(ctx, mem, abi.MIXED)

    def step_sequential(mem):
        for m in mem:
            m.st_thermal, m.st_darcy = api.step_hrl(ctx, m.Tc_ex, m.Pc_ex, m.ktv, m.kfv, m.Vx, m.Vy, m.Vz, m.params,
                                                    abi.MIXED)

    res = {"members": len(base), "steps": a.ens_steps, "seed": 4,
           "cells_total": int(sum(int(np.prod([s - 2 for s in T.shape])) for T, *_ in base)),
           "unit": "cell-updates/s", "form": "mixed"}
    arms = {}
    with torch.cuda.stream(stream):
        for name, fn in (("batched", step_batched), ("sequential", step_sequential)):
            mem = make()
            fn(mem)  # warm-up: scratch, block-size tuning, graph capture
            reset(mem)
            torch.cuda.synchronize()
            l0 = ctx.launches
            upd = 0
            t0 = time.perf_counter()
            for _ in range(a.ens_steps):
                fn(mem)
                for m in mem:
                    nc = (m.Tc_ex.shape[0] - 2) * (m.Tc_ex.shape[1] - 2) * (m.Tc_ex.shape[2] - 2)
                    upd += nc * (m.st_thermal.iters + m.st_darcy.iters)
            torch.cuda.synchronize()
            t = time.perf_counter() - t0
            arms[name] = dict(mem=mem, t=t, upd=upd, launches=ctx.launches - l0)
            res[name] = {"value": upd / t, "seconds": t, "gpu_launches": ctx.launches - l0}
    res["speedup_batched_vs_sequential"] = res["batched"]["value"] / res["sequential"]["value"]
    res["bitwise_equal"] = bool(all(torch.equal(x.Tc_ex, y.Tc_ex) and torch.equal(x.Pc_ex, y.Pc_ex)
                                    for x, y in zip(arms["batched"]["mem"], arms["sequential"]["mem"])))
    res["same_work"] = arms["batched"]["upd"] == arms["sequential"]["upd"]
    res["block_size"] = "autotuned (HT3D_TUNE_ENS_BLOCK = 0)"
    return res


def sweep_bench(ctx, stream, n, reps=3):
    """One SSP-RK2 WENO5 sweep over the three axes of an n^3 grid (blob in a
    divergence-free curl velocity, CFL 0.5), FP32, mixed and FP64; inputs
    resident in HBM (each field > L2); CUDA events on the ctx stream."""
    import torch
    import hydrothermal3d_gb300 as ht
    from hydrothermal3d_gb300 import api, abi, sweep
    V = sweep.curl_velocity(n, n, n, seed=6)
    T0 = sweep.blob(n, n, n)
    torch.cuda.synchronize()  # built on torch's stream; the sweeps run on the ctx stream
    dt = sweep.cfl_dt(n, n, n, cfl=0.5)
    h = (float(n),) * 3
    bc, bv = [0, 0, 1, 1, 0, 0], [0, 0, 1.0, 0.0, 0, 0]
    res = {"n": n, "velocity": "discrete curl of seeded sine modes (seed 6), max|V| = 1", "cfl": 0.5,
           "unit": "GB/s (21 N s per sweep)"}
    peak = measured_peak()[0]
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        for name, prec, s in (("fp32", None, 4), ("mixed", abi.MIXED, 8), ("fp64", abi.FP64, 8)):
            if prec is None:
                T = T0.float().permute(2, 1, 0).contiguous().permute(2, 1, 0)
                Vs = [v.float().permute(2, 1, 0).contiguous().permute(2, 1, 0) for v in V]
                fn = lambda: api.weno5_advect_f32(ctx, T, *Vs, dt, *h, bc, bv, abi.WENO_V1)
            else:
                T = T0.clone()
                fn = lambda: api.weno5_advect(ctx, T, *V, dt, *h, bc, bv, abi.WENO_V1, prec)
            fn()
            torch.cuda.synchronize()
            e0.record(stream)
            for _ in range(reps):
                fn()
            e1.record(stream)
            torch.cuda.synchronize()
            t = e0.elapsed_time(e1) / 1e3 / reps
            gbs = sweep.bytes_per_sweep(n, n, n, s) / t / 1e9
            res[name] = {"ms_per_sweep": t * 1e3, "T_eff_GBs": gbs, "frac_of_measured_hbm": gbs / peak,
                         "storage_bytes": s}
            del T
    return res


def growth_bench(ctx, stream, steps, n=127, eps=1e-8):
    """How the HRL workload amplifies small differences: per time step, the
    max-norm relative T difference against the FP64 run of (a) the mixed form
    and (b) the FP64 form started from the initial condition perturbed by
    eps * U(-1, 1) (relative, seed 9).  Both use the FP64 run's dt sequence."""
    import torch
    import hydrothermal3d_gb300 as ht
    from hydrothermal3d_gb300 import api, abi, hrl
    T0, P0, ktv, kfv = hrl.initial_fields(n, n, n, seed=1)
    Tp = T0.copy(order="F")
    Tp[1:-1, 1:-1, 1:-1] *= 1.0 + eps * np.random.default_rng(9).uniform(-1, 1, (n, n, n))
    ktd, kfd = ht.from_numpy(ktv), ht.from_numpy(kfv)
    V = [ht.zeros(n + 1, n, n), ht.zeros(n, n + 1, n), ht.zeros(n, n, n + 1)]
    runs = {"fp64": (T0, abi.FP64), "mixed": (T0, abi.MIXED), "fp64_perturbed": (Tp, abi.FP64)}
    fields = {k: (ht.from_numpy(t), ht.from_numpy(P0)) for k, (t, _) in runs.items()}
    inner = (slice(1, -1),) * 3
    out = {"n": n, "perturbation": eps, "mixed_vs_fp64": [], "fp64_perturbed_vs_fp64": []}
    p = hrl.params(n, n, n)
    with torch.cuda.stream(stream):
        for _ in range(steps):
            dt = p.dt
            api.step_hrl(ctx, *fields["fp64"], ktd, kfd, *V, p, abi.FP64)
            for k in ("mixed", "fp64_perturbed"):
                q = hrl.params(n, n, n)
                q.dt = dt
                api.step_hrl(ctx, *fields[k], ktd, kfd, *V, q, runs[k][1])
            torch.cuda.synchronize()
            ref = fields["fp64"][0][inner]
            scale = float(ref.abs().max())
            out["mixed_vs_fp64"].append(float((fields["mixed"][0][inner] - ref).abs().max()) / scale)
            out["fp64_perturbed_vs_fp64"].append(float((fields["fp64_perturbed"][0][inner] - ref).abs().max()) / scale)
    out["note"] = ("a 1e-8 perturbation of the FP64 run grows like the mixed form's difference: the accumulated "
                   "difference measures the convective instability of the workload, the per-step error the form")
    return out


def accuracy_bench(ctx, stream, steps, n=255, cadence=500, out_path="", eps=1e-8):
    """The mixed form's error against the FP64 form over `steps` HRL time steps
    at n^3 (Ra 1000, tolerance 1e-8, seed-1 initial condition), every run
    forced onto the FP64 run's dt sequence.  Per step, the max-norm relative
    difference of T, P (mean removed) and the Darcy velocities Vx, Vy, Vz
    against the FP64 run, for:
      local      one mixed step taken from the FP64 state of the step before
                 (the error the mixed form adds in one step);
      mixed      the mixed run from the initial condition (accumulated);
      perturbed  an FP64 run from the initial condition perturbed by
                 eps * U(-1, 1) relative (seed 9);
      cadence    an FP64 run that tests convergence every `cadence`
                 pseudo-iterations instead of 1000: another FP64 answer that
                 meets the same tolerance.
    The two FP64 controls measure how far the workload itself carries a
    difference of the size the solver tolerance leaves."""
    import torch
    import hydrothermal3d_gb300 as ht
    from hydrothermal3d_gb300 import api, abi, hrl
    T0, P0, ktv, kfv = hrl.initial_fields(n, n, n, seed=1)
    Tp = T0.copy(order="F")
    Tp[1:-1, 1:-1, 1:-1] *= 1.0 + eps * np.random.default_rng(9).uniform(-1, 1, (n, n, n))
    ktd, kfd = ht.from_numpy(ktv), ht.from_numpy(kfv)

    def vel():
        return [ht.zeros(n + 1, n, n), ht.zeros(n, n + 1, n), ht.zeros(n, n, n + 1)]

    runs = {"fp64": (T0, abi.FP64, 1000), "mixed": (T0, abi.MIXED, 1000), "perturbed": (Tp, abi.FP64, 1000)}
    if cadence:
        runs["cadence"] = (T0, abi.FP64, cadence)
    state = {k: [ht.from_numpy(t), ht.from_numpy(P0)] + vel() for k, (t, _, _) in runs.items()}
    local = [ht.zeros(n + 2, n + 2, n + 2), ht.zeros(n + 2, n + 2, n + 2)] + vel()
    inner = (slice(1, -1),) * 3
    names = ("T", "P", "Vx", "Vy", "Vz")

    def errors(s, r):
        e = {}
        for nm, x, y in zip(names, s, r):
            if nm == "T":
                x, y = x[inner], y[inner]
            elif nm == "P":
                x, y = x[inner] - x[inner].mean(), y[inner] - y[inner].mean()
            e[nm] = float((x - y).abs().max() / y.abs().max())
        return e

    rec = {"n": n, "steps": steps, "tolerance": 1e-8, "perturbation": eps, "cadence_control_nitout": cadence,
           "per_step": []}
    p = hrl.params(n, n, n)
    t_start = time.perf_counter()
    with torch.cuda.stream(stream):
        torch.cuda.synchronize()
        for k in range(steps):
            dt = p.dt
            for dst, src in zip(local, state["fp64"]):
                dst.copy_(src)
            f = state["fp64"]
            gt, gd = api.step_hrl(ctx, f[0], f[1], ktd, kfd, *f[2:], p, abi.FP64)
            row = {"step": k + 1, "dt": dt, "iters_fp64": [gt.iters, gd.iters]}
            q = hrl.params(n, n, n)
            q.dt = dt
            lt, ld = api.step_hrl(ctx, local[0], local[1], ktd, kfd, *local[2:], q, abi.MIXED)
            row["iters_local"] = [lt.iters, ld.iters]
            for key in runs:
                if key == "fp64":
                    continue
                q = hrl.params(n, n, n, nitout=runs[key][2])
                q.dt = dt
                s = state[key]
                st, sd = api.step_hrl(ctx, s[0], s[1], ktd, kfd, *s[2:], q, runs[key][1])
                row["iters_" + key] = [st.iters, sd.iters]
            torch.cuda.synchronize()
            ref = state["fp64"]
            row["local"] = errors(local, ref)
            for key in runs:
                if key != "fp64":
                    row[key] = errors(state[key], ref)
            T = ref[0][inner]
            row["T_range"] = [float(T.min()), float(T.max())]
            row["max_abs_V"] = max(float(v.abs().max()) for v in ref[2:])
            rec["per_step"].append(row)
            print(json.dumps({"accuracy_step": row}), file=sys.stderr, flush=True)
    rec["seconds"] = time.perf_counter() - t_start
    ps = rec["per_step"]
    rec["max_local"] = {nm: max(r["local"][nm] for r in ps) for nm in names}
    for key in runs:
        if key != "fp64":
            rec["final_" + key] = ps[-1][key]
    if out_path:
        with open(out_path, "w") as f:
            json.dump(rec, f)
    return rec


def v18_bench(ctx, stream, steps, n=127, nitmax=100000):
    """Dimensional model (ht3d_step_v18, plain FP64) on the 10 x 10 x 5 km box
    at n^3: the steady initialisation step (it = 0) and the following steps
    with pluton insertion and WENO5-v2 sub-stepping, DYREL tolerance 1e-10.
    T_eff counts 10N*8+N bytes per thermal and 11N*8+N per Darcy
    pseudo-iteration plus 21N*8 per advection sub-step."""
    import torch
    import hydrothermal3d_gb300 as ht
    from hydrothermal3d_gb300 import api, v18
    b = v18.box(n, n, n, seed=2, nitmax=nitmax)
    p = b["params"]
    T, P = ht.from_numpy(b["T"]), ht.from_numpy(b["P"])
    args = (ht.from_numpy(b["phc"]), ht.from_numpy(b["phv"]), ht.from_numpy(b["wN"]), ht.from_numpy(b["kmul"]))
    V = [ht.zeros(n + 1, n, n), ht.zeros(n, n + 1, n), ht.zeros(n, n, n + 1)]
    bt, bd = v18.bytes_per_iteration(n, n, n)
    rows, nbytes = [], 0
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        torch.cuda.synchronize()
        e0.record(stream)
        for it in range(steps):
            p.it = it
            gt, gd = api.step_v18(ctx, T, P, *args, *V, p)
            rows.append({"it": it, "iters": [gt.iters, gd.iters], "converged": [gt.converged, gd.converged],
                         "nF_rel": [gt.nF_rel, gd.nF_rel], "advection_substeps": p.n_adv})
            nbytes += gt.iters * bt + gd.iters * bd + p.n_adv * 21 * n ** 3 * 8
        e1.record(stream)
        torch.cuda.synchronize()
    t = e0.elapsed_time(e1) / 1e3
    iters = sum(sum(r["iters"]) for r in rows)
    return {"n": n, "steps": steps, "seconds": t, "time_steps_per_s": steps / t, "T_eff_GBs": nbytes / t / 1e9,
            "cell_updates_per_s": iters * n ** 3 / t, "all_converged": all(all(r["converged"]) for r in rows),
            "per_step": rows, "dtype": "f64",
            "case": "10x10x5 km box, T 600->20 C, log10 k ~ N(-15, 0.5) with 500 m correlation (seed 2), "
                    f"DYREL tol 1e-10 relative, nitmax {nitmax}, WENO5 v2 with the reference's stencil, CFL 0.5"}


def c127_bench(ctx, stream, steps, n=127, nitmax=100000):
    """The first `steps` time steps of the 127^3 dimensional box on the oracle
    (C++ FP64, OpenMP over the host cores) and on the GPU's FP64 form: the
    iteration counts and the max-norm relative difference of T, P and the
    Darcy velocities after each step."""
    import torch
    import oracle
    import hydrothermal3d_gb300 as ht
    from hydrothermal3d_gb300 import api, v18
    oracle.set_threads(os.cpu_count())
    b = v18.box(n, n, n, seed=2, nitmax=nitmax)
    q = v18.box(n, n, n, seed=2, nitmax=nitmax)["params"]
    p = b["params"]
    T, P = b["T"].copy(order="F"), b["P"].copy(order="F")
    V = [np.zeros(s, order="F") for s in ((n + 1, n, n), (n, n + 1, n), (n, n, n + 1))]
    Td, Pd = ht.from_numpy(T), ht.from_numpy(P)
    Vd = [ht.zeros(*v.shape) for v in V]
    args = (ht.from_numpy(b["phc"]), ht.from_numpy(b["phv"]), ht.from_numpy(b["wN"]), ht.from_numpy(b["kmul"]))
    inner = (slice(1, -1),) * 3
    rows = []
    t_oracle = 0.0
    for it in range(steps):
        p.it = q.it = it
        with torch.cuda.stream(stream):
            gt, gd = api.step_v18(ctx, Td, Pd, *args, *Vd, q)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s, ot, od = oracle.step_v18(T, P, b["phc"], b["phv"], b["wN"], b["kmul"], *V, p)
        t_oracle += time.perf_counter() - t0
        rel = lambda a, c: float(np.abs(a - c).max() / np.abs(c).max())
        Tg, Pg = ht.to_numpy(Td), ht.to_numpy(Pd)
        rows.append({"it": it, "iters_gpu": [gt.iters, gd.iters], "iters_oracle": [ot.iters, od.iters],
                     "T_rel_err": rel(Tg[inner], T[inner]), "P_rel_err": rel(Pg[inner], P[inner]),
                     "V_rel_err": max(rel(ht.to_numpy(a), c) for a, c in zip(Vd, V)),
                     "T_bitwise": bool(np.array_equal(Tg, T)), "P_bitwise": bool(np.array_equal(Pg, P)),
                     "dt_equal": q.dt == p.dt, "n_adv": [q.n_adv, p.n_adv]})
        print(json.dumps({"config_127_step": rows[-1]}), file=sys.stderr, flush=True)
    return {"n": n, "steps": steps, "per_step": rows, "oracle_seconds": t_oracle, "oracle_cores": oracle.num_threads(),
            "case": "10x10x5 km box (seed 2), DYREL tol 1e-10, nitmax %d, WENO5 v2 (reference stencil)" % nitmax}


def post_bench(ctx, stream, n, reps=5):
    """Output diagnostics of the v18 VTK step at n^3: the reference's ten
    kernels one after another against the fused single pass (bit-identical
    fields), and the Nusselt reduction.  Inputs and outputs (4 GB at 255^3)
    exceed L2."""
    import torch
    from hydrothermal3d_gb300 import api, post
    d = post.device_case(n, n, n, seed=3)
    o = post.outputs(n, n, n)
    qy = d["Vy"]
    torch.cuda.synchronize()  # inputs were built on torch's stream

    def timed(fn):
        fn()
        fn()
        ctx.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    t_sep = timed(lambda: post.run_separate(ctx, d, o))
    t_fus = timed(lambda: post.run_fused(ctx, d, o))
    # one field at a time through the fused kernel: which law costs what
    per_field = {}
    for name in ("phase", "pressure", "temperature", "k_thermal", "heat_capacity", "permeability", "density",
                 "viscosity", "peclet"):
        per_field[name] = timed(lambda: post.run_fused(ctx, d, {name: o[name]}))
    per_field["velocity"] = timed(lambda: post.run_fused(ctx, d, {k: o[k] for k in ("vx", "vy", "vz")}))
    t_nu = timed(lambda: api.Nusselt(ctx, qy, 1.0, 1.0))
    bs, bf = post.bytes_separate(n, n, n), post.bytes_fused(n, n, n)
    return {"n": n, "separate_ms": t_sep, "fused_ms": t_fus, "fused_speedup": t_sep / t_fus,
            "separate_alg_GBs": bs / t_sep / 1e6, "fused_alg_GBs": bf / t_fus / 1e6, "nusselt_ms": t_nu,
            "single_field_ms": per_field, "alg_bytes_per_cell": {"separate": bs // n ** 3, "fused": bf // n ** 3}, "dtype": "f64",
            "case": "seeded phases (crust, fault, pluton, immersed, 5 % air rows), T 300-900 K, P 0.1-300 MPa, "
                    "face velocities; all twelve VTK fields"}


def nusselt_bench(ctx, stream, steps, n=63):
    """Nusselt-number time series of the HRL run at n^3 through the time-loop
    driver, plain FP64 and mixed form from the same initial state: the mixed
    form must track the FP64 physics over many steps."""
    import torch
    import hydrothermal3d_gb300 as ht
    from hydrothermal3d_gb300 import abi, driver, hrl
    out = {"n": n, "steps": steps}
    series = {}
    with torch.cuda.stream(stream):
        for name, prec in (("fp64", abi.FP64), ("mixed", abi.MIXED)):
            T0, P0, ktv, kfv = hrl.initial_fields(n, n, n, seed=1)
            T, P, ktd, kfd = (ht.from_numpy(x) for x in (T0, P0, ktv, kfv))
            V = (ht.zeros(n + 1, n, n), ht.zeros(n, n + 1, n), ht.zeros(n, n, n + 1))
            p = hrl.params(n, n, n)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            recs = driver.run_hrl(ctx, T, P, ktd, kfd, V, p, steps, prec)
            out[name + "_seconds"] = time.perf_counter() - t0
            series[name] = [(r["time"], r["Nu"]) for r in recs]
    nu64 = [nu for _, nu in series["fp64"]]
    numx = [nu for _, nu in series["mixed"]]
    out["Nu_fp64_every_10_steps"] = nu64[9::10]
    out["Nu_mixed_every_10_steps"] = numx[9::10]
    out["time_every_10_steps"] = [t for t, _ in series["fp64"]][9::10]
    out["max_abs_Nu_difference"] = max(abs(x - y) for x, y in zip(nu64, numx))
    out["note"] = "Nu of T after each step (driver.py); both runs from the seed-1 initial condition"
    return out


def fault_bench(ctx, stream, a):
    """511^3 mixed-form HRL steps with a log-normal permeability and a x10
    fault slab (seed 5)."""
    import torch
    import hydrothermal3d_gb300 as ht
    from hydrothermal3d_gb300 import api, abi, hrl
    n = 511
    T, P, ktv, kfv, p = hrl.fault_slab_case(n=n, seed=5)
    V = [ht.zeros(n + 1, n, n), ht.zeros(n, n + 1, n), ht.zeros(n, n, n + 1)]
    iters, nbytes = [], 0
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(a.fault_steps):
            gt, gd = api.step_hrl(ctx, T, P, ktv, kfv, *V, p, abi.MIXED)
            iters.append((gt.iters, gd.iters))
            nbytes += (gt.iters + gd.iters) * hrl.bytes_per_iteration(n, n, n, 4) + hrl.bytes_per_advection(n, n, n, 4)
        e1.record(stream)
        torch.cuda.synchronize()
    t = e0.elapsed_time(e1) / 1e3
    inner = T[1:-1, 1:-1, 1:-1]
    return {"n": n, "steps": a.fault_steps, "seconds": t, "time_steps_per_s": a.fault_steps / t,
            "T_eff_GBs": nbytes / t / 1e9, "pseudo_iterations_per_step": [list(x) for x in iters],
            "T_range": [float(inner.min()), float(inner.max())], "dt_last": p.dt,
            "case": "HRL Ra 1000, log-normal kf (log10 sigma 0.25, 4-cell correlation) with a x10 slab 3 cells "
                    "wide at mid-x, seed 5, dt_max 1e-3, mixed form, no warm-up (first steps from the initial "
                    "condition)"}


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs)"
    except Exception:
        return 6800.0, "fallback 6.8 TB/s"


def profile_traffic(name):
    """DRAM bytes per pseudo-iteration at 255^3 from the committed ncu summary
    (a line 'traffic_bytes_per_iteration_at_255: B'), if one exists."""
    p = os.path.join(ROOT, "profiles", f"{name}.md")
    try:
        with open(p) as f:
            for line in f:
                if line.startswith("traffic_bytes_per_iteration_at_255:"):
                    return float(line.split(":", 1)[1].split()[0])
    except Exception:
        pass
    return None


def main():
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)


if __name__ == "__main__":
    main()
