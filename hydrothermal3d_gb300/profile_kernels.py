"""Run one hot kernel of libht3d in isolation, for timing and ncu captures.

  python -m hydrothermal3d_gb300.profile_kernels --kernel dyrel_f32 --n 255 --iters 5
  ncu --set full --clock-control none -k regex:k_dyrel_iter -s 2 -c 1 -o out \\
      python -m hydrothermal3d_gb300.profile_kernels --kernel dyrel_f32 --n 255 --iters 5

Kernels: weno_f32 (one FP32 WENO5 sweep in a curl velocity),
dyrel_f32 (FP32 pseudo-iteration on the reference layout),
dyrel_f64 (plain FP64 pseudo-iteration), mixed_solve (a mixed-form DYREL
solve of --iters pseudo-iterations: two FP64 checks, then the padded FP32
inner iterations, two per pass in k_mixed_inner2, or one per launch in
k_mixed_inner with --tune 6=0), weno_f64 / weno_mixed (one fused WENO5
advection), post (one fused pass of the twelve output diagnostics, k_post),
dim_step (one dimensional v18 time step, it = 0, with --iters pseudo-iterations
per solve: k_dim_iter thermal then Darcy).
Prints the average time per launch measured with CUDA events.
"""
import argparse
import json

import torch

import hydrothermal3d_gb300 as ht
from hydrothermal3d_gb300 import abi, hrl


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--kernel", default="dyrel_f32",
                    choices=["dyrel_f32", "dyrel_f64", "mixed_solve", "weno_f64", "weno_mixed", "weno_f32",
                             "ensemble", "post", "dim_step"])
    ap.add_argument("--members", type=int, default=16, help="ensemble members (--kernel ensemble)")
    ap.add_argument("--n", type=int, default=255)
    ap.add_argument("--iters", type=int, default=5)
    ap.add_argument("--variant", type=int, default=0,
                    help="DYREL thread layout: 0 per precision, 1 z-march tiles, 2 one thread per cell")
    ap.add_argument("--tune", action="append", default=[],
                    help="KEY=VALUE context tuning (HT3D_TUNE_* number), repeatable")
    a = ap.parse_args()
    n = a.n
    stream = torch.cuda.Stream()
    ctx = ht.Context(device=0, stream=stream.cuda_stream)
    ctx.check(ctx.lib.ht3d_ctx_set_tuning(ctx.ptr, abi.TUNE_DYREL_VARIANT, a.variant))
    for kv in a.tune:
        key, val = (int(x) for x in kv.split("="))
        ctx.set_tuning(key, val)
    d = 1.0 / n
    bt, bv = abi.int6(0, 0, 1, 1, 0, 0), abi.dbl6(0, 0, 1, 0, 0, 0)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if a.kernel.startswith("dyrel"):
        dt = torch.float32 if a.kernel == "dyrel_f32" else torch.float64
        X = ht.zeros(n + 2, n + 2, n + 2, dtype=dt).uniform_(0, 1)
        R = ht.zeros(n, n, n, dtype=dt).uniform_(-1, 1)
        k = [ht.ones(n + 1, n, n, dtype=dt), ht.ones(n, n + 1, n, dtype=dt), ht.ones(n, n, n + 1, dtype=dt)]
        pc = 6.0 * n * n
        PCx = ht.ones(n, n, n, dtype=dt) * (1.0 / pc if a.kernel == "dyrel_f32" else pc)
        F0 = ht.zeros(n, n, n, dtype=dt)
        name = "ht3d_dyrel_iterate_f32" if a.kernel == "dyrel_f32" else "ht3d_dyrel_iterate"
        torch.cuda.synchronize()  # inputs were built on torch's stream
        args = lambda m: (X.data_ptr(), R.data_ptr(), k[0].data_ptr(), k[1].data_ptr(), k[2].data_ptr(),
                          PCx.data_ptr(), F0.data_ptr(), 0.0, d, d, d, bt, bv, 0.99, 0.05, 0.01, m, n, n, n)
        torch.cuda.synchronize()
        ctx.call(name, *args(2))
        ctx.synchronize()
        e0.record(stream)
        ctx.call(name, *args(a.iters))
        e1.record(stream)
        torch.cuda.synchronize()
        t = e0.elapsed_time(e1) / 1e3 / a.iters
        s = 4 if a.kernel == "dyrel_f32" else 8
        alg = hrl.bytes_per_iteration(n, n, n, s)
        print(json.dumps({"kernel": a.kernel, "variant": a.variant, "n": n, "us_per_launch": t * 1e6, "alg_GBs": alg / t / 1e9}))
    elif a.kernel == "mixed_solve":
        from hydrothermal3d_gb300 import api
        X = ht.zeros(n + 2, n + 2, n + 2).uniform_(0, 1)
        R = ht.zeros(n, n, n).uniform_(-1, 1)
        k = [ht.ones(n + 1, n, n), ht.ones(n, n + 1, n), ht.ones(n, n, n + 1)]
        F, F0 = ht.zeros(n, n, n), ht.zeros(n, n, n)
        prm = abi.DyrelParams.reference()
        ctx.set_tuning(abi.TUNE_TIME_INNER, 1)
        torch.cuda.synchronize()  # inputs were built on torch's stream
        with torch.cuda.stream(stream):
            api.dyrel_solve_dimless(ctx, X, R, *k, float(n * n), d, d, d, (0, 0, 1, 1, 0, 0), (0, 0, 1, 0, 0, 0), prm,
                                    F, F0, abi.MIXED, n_iter_fixed=a.iters)
        torch.cuda.synchronize()
        ms, nl = ctx.inner_timing(reset=True)
        t = ms / 1e3 / max(1, nl)
        alg = hrl.bytes_per_iteration(n, n, n, 4)
        single = any(kv.replace(" ", "") == f"{abi.TUNE_TEMPORAL}=0" for kv in a.tune)
        print(json.dumps({"kernel": "k_mixed_inner" if single else "k_mixed_inner2 (two iterations per pass)",
                          "n": n, "tune": a.tune, "inner_iterations": nl,
                          "us_per_iteration": t * 1e6, "alg_GBs": alg / t / 1e9}))
    elif a.kernel == "ensemble":
        from hydrothermal3d_gb300 import api
        mem = []
        for T, P, ktv, kfv, p in hrl.ensemble(a.members, seed=4):
            nx, ny, nz = (q - 2 for q in T.shape)
            mem.append(api.Member(ht.from_numpy(T), ht.from_numpy(P), ht.from_numpy(ktv), ht.from_numpy(kfv),
                                  ht.zeros(nx + 1, ny, nz), ht.zeros(nx, ny + 1, nz), ht.zeros(nx, ny, nz + 1), p))
        ctx.set_tuning(abi.TUNE_TIME_INNER, 1)
        torch.cuda.synchronize()  # inputs were built on torch's stream
        with torch.cuda.stream(stream):
            for _ in range(a.iters):
                api.ensemble_step(ctx, mem, abi.MIXED)
        torch.cuda.synchronize()
        ms, nl = ctx.inner_timing(reset=True)
        cells = sum(int(m.Tc_ex.shape[0] - 2) * int(m.Tc_ex.shape[1] - 2) * int(m.Tc_ex.shape[2] - 2) for m in mem)
        print(json.dumps({"kernel": "k_ens_inner", "members": len(mem), "cells": cells, "inner_iterations": nl,
                          "us_per_iteration": 1e3 * ms / max(1, nl)}))
    elif a.kernel == "post":
        from hydrothermal3d_gb300 import post
        d = post.device_case(n, n, n, seed=3)
        o = post.outputs(n, n, n)
        torch.cuda.synchronize()  # inputs were built on torch's stream
        post.run_fused(ctx, d, o)
        ctx.synchronize()
        e0.record(stream)
        for _ in range(a.iters):
            post.run_fused(ctx, d, o)
        e1.record(stream)
        torch.cuda.synchronize()
        t = e0.elapsed_time(e1) / 1e3 / a.iters
        print(json.dumps({"kernel": "k_post", "n": n, "us_per_pass": t * 1e6,
                          "alg_GBs": post.bytes_fused(n, n, n) / t / 1e9}))
    elif a.kernel == "dim_step":
        from hydrothermal3d_gb300 import api, v18
        nit = max(2, a.iters)
        b = v18.box(n, n, n, seed=2, nitmax=nit, nitout=max(1, nit // 2))
        p = b["params"]
        p.it = 0
        T, P = ht.from_numpy(b["T"]), ht.from_numpy(b["P"])
        args = (ht.from_numpy(b["phc"]), ht.from_numpy(b["phv"]), ht.from_numpy(b["wN"]), ht.from_numpy(b["kmul"]))
        V = [ht.zeros(n + 1, n, n), ht.zeros(n, n + 1, n), ht.zeros(n, n, n + 1)]
        torch.cuda.synchronize()  # inputs were built on torch's stream
        with torch.cuda.stream(stream):
            e0.record(stream)
            gt, gd = api.step_v18(ctx, T, P, *args, *V, p)
            e1.record(stream)
        torch.cuda.synchronize()
        t = e0.elapsed_time(e1) / 1e3
        bt, bd = v18.bytes_per_iteration(n, n, n)
        print(json.dumps({"kernel": "k_dim_iter (v18 step)", "n": n, "iters": [gt.iters, gd.iters], "ms_per_step": t * 1e3,
                          "alg_GBs_iterations": (gt.iters * bt + gd.iters * bd) / t / 1e9}))
    elif a.kernel == "weno_f32":
        from hydrothermal3d_gb300 import api, sweep
        V = [v.float().permute(2, 1, 0).contiguous().permute(2, 1, 0) for v in sweep.curl_velocity(n, n, n, seed=6)]
        T = sweep.blob(n, n, n).float().permute(2, 1, 0).contiguous().permute(2, 1, 0)
        dtc = sweep.cfl_dt(n, n, n)
        torch.cuda.synchronize()  # inputs were built on torch's stream
        run = lambda: api.weno5_advect_f32(ctx, T, *V, dtc, float(n), float(n), float(n), [0, 0, 1, 1, 0, 0],
                                           [0, 0, 1.0, 0.0, 0, 0], abi.WENO_V1)
        run()
        ctx.synchronize()
        e0.record(stream)
        for _ in range(a.iters):
            run()
        e1.record(stream)
        torch.cuda.synchronize()
        t = e0.elapsed_time(e1) / 1e3 / a.iters
        print(json.dumps({"kernel": "weno_f32 sweep", "n": n, "us_per_sweep": t * 1e6,
                          "alg_GBs": sweep.bytes_per_sweep(n, n, n, 4) / t / 1e9}))
    else:
        prec = abi.FP64 if a.kernel == "weno_f64" else abi.MIXED
        T = ht.zeros(n + 2, n + 2, n + 2).uniform_(0, 1)
        V = [ht.zeros(n + 1, n, n).uniform_(-1, 1), ht.zeros(n, n + 1, n).uniform_(-1, 1), ht.zeros(n, n, n + 1).uniform_(-1, 1)]
        torch.cuda.synchronize()  # inputs were built on torch's stream
        args = (T.data_ptr(), V[0].data_ptr(), V[1].data_ptr(), V[2].data_ptr(), 0.1 * d, float(n), float(n), float(n),
                abi.int6(0, 0, 1, 1, 0, 0), abi.dbl6(0, 0, 1, 0, 0, 0), abi.WENO_V1, prec, n, n, n)
        ctx.call("ht3d_weno5_advect", *args)
        ctx.synchronize()
        e0.record(stream)
        for _ in range(a.iters):
            ctx.call("ht3d_weno5_advect", *args)
        e1.record(stream)
        torch.cuda.synchronize()
        t = e0.elapsed_time(e1) / 1e3 / a.iters
        s = 8 if prec == abi.FP64 else 4
        alg = hrl.bytes_per_advection(n, n, n, s)
        print(json.dumps({"kernel": a.kernel, "n": n, "us_per_advection": t * 1e6, "alg_GBs": alg / t / 1e9}))
    ctx.close()


if __name__ == "__main__":
    main()
