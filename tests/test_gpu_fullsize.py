"""GPU tests at the workloads' full sizes, through properties that hold at any
size.  The oracle checks the same paths bit for bit or to the stated
tolerances at sizes it finishes in seconds (test_gpu_solver.py,
test_gpu_weno_sweep.py, test_gpu_ensemble.py); here the GPU forms are checked
against each other where the oracle would take minutes to hours:

* 255^3 HRL time step (the mixed-form workload): one mixed step and one
  FP64 step from the same seeded state; T within 1e-6 (relative max-norm,
  the mixed form's accuracy target) and P (mean removed) within 1e-6; both
  forms' solves converge.
* 255^3 HRL, six steps on the FP64 trajectory (through the onset of
  convection, where the reference's dt rule takes a CFL-22 advection step):
  at every step one mixed step from the FP64 state with the FP64 run's dt
  stays within 1e-6 of the FP64 step in T and P, with the same iteration
  counts.
* 511^3 WENO5 sweep (blob in the seeded divergence-free curl velocity, CFL
  0.5): the FP32 sweep within 2e-5 and the mixed sweep within 2e-6 of the
  FP64 sweep (relative to max |T|), the per-sweep tolerances of the
  small-size tests.
* the 64-member ensemble at its full member sizes (n ~ U{31..95} per axis,
  seed 4): one batched mixed step is bitwise equal to the members stepped
  one by one.
* the 127^3 dimensional box (FP64): two runs of the steady initialisation
  step and the first step with pluton insertion and WENO5 sub-steps, from
  the same state, agree bit for bit (every sum has a fixed order), with
  finite fields and equal solver statistics."""
import pytest
import torch

import hydrothermal3d_gb300 as ht
from hydrothermal3d_gb300 import api, abi, hrl, sweep, v18

pytestmark = pytest.mark.gpu

INNER = (slice(1, -1),) * 3


def test_hrl_255_mixed_step_tracks_fp64(ctx):
    n = 255
    T, P, ktv, kfv = hrl.initial_fields(n, n, n, seed=1)
    ktd, kfd = ht.from_numpy(ktv), ht.from_numpy(kfv)
    out = {}
    for name, prec in (("fp64", abi.FP64), ("mixed", abi.MIXED)):
        Td, Pd = ht.from_numpy(T), ht.from_numpy(P)
        V = [ht.zeros(n + 1, n, n), ht.zeros(n, n + 1, n), ht.zeros(n, n, n + 1)]
        p = hrl.params(n, n, n)
        gt, gd = api.step_hrl(ctx, Td, Pd, ktd, kfd, *V, p, prec)
        assert gt.status == 0 and gd.status == 0, name
        assert gt.converged and gd.converged, name
        out[name] = (Td, Pd, p.dt)
    ctx.synchronize()
    (T6, P6, dt6), (Tm, Pm, dtm) = out["fp64"], out["mixed"]
    T6, Tm = T6[INNER], Tm[INNER]
    P6, Pm = P6[INNER] - P6[INNER].mean(), Pm[INNER] - Pm[INNER].mean()
    assert torch.isfinite(Tm).all() and torch.isfinite(Pm).all()
    assert float((Tm - T6).abs().max() / T6.abs().max()) <= 1e-6
    assert float((Pm - P6).abs().max() / P6.abs().max()) <= 1e-6
    assert abs(dtm - dt6) <= 1e-6 * dt6  # the next step's dt comes from the velocity of each form


def test_hrl_255_mixed_step_error_on_the_fp64_trajectory(ctx):
    """The error the mixed form adds per time step, over the first six steps
    of the 255^3 workload (the sixth takes the onset step)."""
    n = 255
    T, P, ktv, kfv = hrl.initial_fields(n, n, n, seed=1)
    ktd, kfd = ht.from_numpy(ktv), ht.from_numpy(kfv)
    vel = lambda: [ht.zeros(n + 1, n, n), ht.zeros(n, n + 1, n), ht.zeros(n, n, n + 1)]
    Td, Pd, V = ht.from_numpy(T), ht.from_numpy(P), vel()
    Tl, Pl, Vl = ht.zeros(*Td.shape), ht.zeros(*Pd.shape), vel()
    p = hrl.params(n, n, n)
    errs = []
    for step in range(6):
        ctx.synchronize()
        Tl.copy_(Td)
        Pl.copy_(Pd)
        torch.cuda.synchronize()
        q = hrl.params(n, n, n)
        q.dt = p.dt
        lt, ld = api.step_hrl(ctx, Tl, Pl, ktd, kfd, *Vl, q, abi.MIXED)
        gt, gd = api.step_hrl(ctx, Td, Pd, ktd, kfd, *V, p, abi.FP64)
        assert (lt.iters, ld.iters) == (gt.iters, gd.iters), step
        ctx.synchronize()
        t6, tm = Td[INNER], Tl[INNER]
        p6, pm = Pd[INNER] - Pd[INNER].mean(), Pl[INNER] - Pl[INNER].mean()
        errs.append((float((tm - t6).abs().max() / t6.abs().max()), float((pm - p6).abs().max() / p6.abs().max())))
    assert max(e[0] for e in errs) <= 1e-6, errs
    assert max(e[1] for e in errs) <= 1e-6, errs


def _f32(t):
    return t.float().permute(2, 1, 0).contiguous().permute(2, 1, 0)


def test_weno_sweep_511_precisions_track_fp64(ctx):
    n = 511
    V = sweep.curl_velocity(n, n, n, seed=6)
    T0 = sweep.blob(n, n, n)
    torch.cuda.synchronize()
    dt = sweep.cfl_dt(n, n, n, cfl=0.5)
    h = (float(n),) * 3
    bc, bv = [0, 0, 1, 1, 0, 0], [0, 0, 1.0, 0.0, 0, 0]
    T64 = T0.clone()
    api.weno5_advect(ctx, T64, *V, dt, *h, bc, bv, abi.WENO_V1, abi.FP64)
    Tmx = T0.clone()
    api.weno5_advect(ctx, Tmx, *V, dt, *h, bc, bv, abi.WENO_V1, abi.MIXED)
    T32 = _f32(T0)
    Vs = [_f32(v) for v in V]
    del V
    api.weno5_advect_f32(ctx, T32, *Vs, dt, *h, bc, bv, abi.WENO_V1)
    ctx.synchronize()
    ref = T64[INNER]
    scale = float(ref.abs().max())
    assert torch.isfinite(ref).all()
    assert float((Tmx[INNER] - ref).abs().max()) <= 2e-6 * scale
    assert float((T32[INNER].double() - ref).abs().max()) <= 2e-5 * scale


def _members(base):
    mem = []
    for T, P, ktv, kfv, p in base:
        nx, ny, nz = (s - 2 for s in T.shape)
        mem.append(api.Member(ht.from_numpy(T), ht.from_numpy(P), ht.from_numpy(ktv), ht.from_numpy(kfv),
                              ht.zeros(nx + 1, ny, nz), ht.zeros(nx, ny + 1, nz), ht.zeros(nx, ny, nz + 1),
                              abi.HrlParams.from_buffer_copy(p)))
    return mem


def test_ensemble_full_sizes_batched_bitwise_equals_sequential(ctx):
    base = hrl.ensemble(n_members=64, seed=4)
    assert len(base) == 64 and min(min(s - 2 for s in T.shape) for T, *_ in base) >= 31
    batched, sequential = _members(base), _members(base)
    api.ensemble_step(ctx, batched, abi.MIXED)
    for m in sequential:
        m.st_thermal, m.st_darcy = api.step_hrl(ctx, m.Tc_ex, m.Pc_ex, m.ktv, m.kfv, m.Vx, m.Vy, m.Vz, m.params,
                                                abi.MIXED)
    ctx.synchronize()
    for x, y in zip(batched, sequential):
        for f in ("Tc_ex", "Pc_ex", "Vx", "Vy", "Vz"):
            assert torch.equal(getattr(x, f), getattr(y, f)), f
        assert x.params.dt == y.params.dt
        assert x.st_thermal.iters == y.st_thermal.iters and x.st_darcy.iters == y.st_darcy.iters


def test_v18_127_steps_are_reproducible(ctx):
    n = 127
    b = v18.box(n, n, n, seed=2, nitmax=2000)
    args = (ht.from_numpy(b["phc"]), ht.from_numpy(b["phv"]), ht.from_numpy(b["wN"]), ht.from_numpy(b["kmul"]))
    runs = []
    for _ in range(2):
        p = abi.V18Params.from_buffer_copy(b["params"])
        T, P = ht.from_numpy(b["T"]), ht.from_numpy(b["P"])
        V = [ht.zeros(n + 1, n, n), ht.zeros(n, n + 1, n), ht.zeros(n, n, n + 1)]
        stats = []
        for it in range(2):
            p.it = it
            gt, gd = api.step_v18(ctx, T, P, *args, *V, p)
            stats.append((gt.iters, gd.iters, gt.status, gd.status, gt.nF_abs, gd.nF_abs, p.n_adv, p.dt))
        ctx.synchronize()
        runs.append((T, P, V, stats))
    (T1, P1, V1, s1), (T2, P2, V2, s2) = runs
    assert s1 == s2
    assert s1[1][6] > 0  # the second step advected
    assert torch.isfinite(T1).all() and torch.isfinite(P1).all()
    assert torch.equal(T1, T2) and torch.equal(P1, P2)
    for a, c in zip(V1, V2):
        assert torch.equal(a, c)

