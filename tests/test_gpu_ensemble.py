"""Batched ensemble step (ht3d_ensemble_step) against the same members stepped
one by one with ht3d_step_hrl.  The batched mixed solve runs the members'
pseudo-iterations in lockstep (one launch over all members, CUDA-graph windows,
tuned tile shape) but every kernel, schedule and reduction of a member is the
single-instance one: the results must agree bit for bit."""
import numpy as np
import pytest
import torch

import hydrothermal3d_gb300 as ht
from hydrothermal3d_gb300 import api, abi, hrl

pytestmark = pytest.mark.gpu

SIZES = [(7, 9, 5), (16, 12, 8), (33, 17, 9), (31, 32, 30), (5, 40, 6)]


def members_np(sizes=SIZES, seed=41, nitout=100):
    rng = np.random.default_rng(seed)
    out = []
    for m, (nx, ny, nz) in enumerate(sizes):
        T, P, ktv, _ = hrl.initial_fields(nx, ny, nz, seed=seed + m, amp=1e-2)
        kfv = np.asfortranarray(10.0 ** rng.normal(0.0, 0.2, (nx + 1, ny + 1, nz + 1)))
        p = hrl.params(nx, ny, nz, Ra=float(rng.uniform(200, 2000)), nitout=nitout, nitmax=4000,
                       dt_max=2e-4 if m % 2 else 0.0)
        out.append((T, P, ktv, kfv, p))
    return out


def to_device(members):
    res = []
    for T, P, ktv, kfv, p in members:
        nx, ny, nz = (s - 2 for s in T.shape)
        q = abi.HrlParams.from_buffer_copy(p)
        res.append(api.Member(ht.from_numpy(T), ht.from_numpy(P), ht.from_numpy(ktv), ht.from_numpy(kfv),
                              ht.zeros(nx + 1, ny, nz), ht.zeros(nx, ny + 1, nz), ht.zeros(nx, ny, nz + 1), q))
    return res


def step_sequential(ctx, mem, precision):
    for m in mem:
        m.st_thermal, m.st_darcy = api.step_hrl(ctx, m.Tc_ex, m.Pc_ex, m.ktv, m.kfv, m.Vx, m.Vy, m.Vz, m.params,
                                                precision)


def assert_same(a, b):
    for x, y in zip(a, b):
        for f in ("Tc_ex", "Pc_ex", "Vx", "Vy", "Vz"):
            np.testing.assert_array_equal(ht.to_numpy(getattr(x, f)), ht.to_numpy(getattr(y, f)), err_msg=f)
        assert x.params.dt == y.params.dt
        for s, t in ((x.st_thermal, y.st_thermal), (x.st_darcy, y.st_darcy)):
            assert s.iters == t.iters and s.checks == t.checks and s.converged == t.converged
            assert s.nF_abs == t.nF_abs and s.h1 == t.h1 and s.lambda_min == t.lambda_min


@pytest.fixture
def tuned(ctx):
    ctx.set_tuning(abi.TUNE_MIXED_REFRESH, 64)
    yield ctx
    ctx.set_tuning(abi.TUNE_MIXED_REFRESH, 512)
    ctx.set_tuning(abi.TUNE_ENS_BLOCK, 0)
    ctx.set_tuning(abi.TUNE_ENS_TILE, 0)
    ctx.set_tuning(abi.TUNE_ENS_GRAPH, 1)


# tile shapes: 0 = autotuned; 1-3 one plane per thread (64/128/256 threads),
# 4-6 z-marching threads (64x8, 128x8, 128x16 planes); a block size alone
# selects the one-plane kernel
@pytest.mark.parametrize("block,tile,graphs", [(0, 0, 1), (64, 0, 0), (128, 0, 1), (256, 0, 0), (0, 4, 1),
                                               (0, 5, 0), (0, 6, 1)])
def test_ensemble_mixed_bitwise_equals_sequential(tuned, block, tile, graphs):
    ctx = tuned
    ctx.set_tuning(abi.TUNE_ENS_BLOCK, block)
    ctx.set_tuning(abi.TUNE_ENS_TILE, tile)
    ctx.set_tuning(abi.TUNE_ENS_GRAPH, graphs)
    base = members_np()
    seq, ens = to_device(base), to_device(base)
    l0 = ctx.launches
    for _ in range(2):
        step_sequential(ctx, seq, abi.MIXED)
    l1 = ctx.launches
    for _ in range(2):
        assert api.ensemble_step(ctx, ens, abi.MIXED) == [abi.OK] * len(ens)
    l2 = ctx.launches
    torch.cuda.synchronize()
    assert_same(ens, seq)
    assert all(m.st_thermal.converged and m.st_darcy.converged for m in ens)
    # one launch per lockstep pseudo-iteration instead of one per member
    assert l2 - l1 < l1 - l0


def test_ensemble_tile_shape_changes_between_steps(tuned):
    """Consecutive solves with different tile shapes (their CUDA graphs are
    keyed by the launch groups' version and the shape): every step stays bit
    for bit equal to the per-member steps."""
    ctx = tuned
    base = members_np(SIZES[:3])
    seq, ens = to_device(base), to_device(base)
    for tile in (1, 4, 2, 5, 3, 6, 0):
        ctx.set_tuning(abi.TUNE_ENS_TILE, tile)
        step_sequential(ctx, seq, abi.MIXED)
        assert api.ensemble_step(ctx, ens, abi.MIXED) == [abi.OK] * len(ens)
        torch.cuda.synchronize()
        assert_same(ens, seq)


def test_ensemble_fp64_equals_sequential(ctx):
    base = members_np(SIZES[:3], nitout=50)
    seq, ens = to_device(base), to_device(base)
    step_sequential(ctx, seq, abi.FP64)
    api.ensemble_step(ctx, ens, abi.FP64)
    assert_same(ens, seq)


def test_ensemble_member_failure_is_isolated(tuned):
    ctx = tuned
    base = members_np(SIZES[:3])
    T = base[1][0].copy(order="F")
    T[3, 3, 3] = np.nan
    base[1] = (T,) + base[1][1:]
    seq, ens = to_device(base), to_device(base)
    with pytest.raises(ht.Ht3dError):
        api.ensemble_step(ctx, ens, abi.MIXED)
    assert [m.status for m in ens] == [abi.OK, abi.ERR_NAN, abi.OK]
    for i in (0, 2):
        step_sequential(ctx, seq[i:i + 1], abi.MIXED)
    assert_same([ens[0], ens[2]], [seq[0], seq[2]])


def test_ensemble_requires_shared_schedule(ctx):
    base = members_np(SIZES[:2])
    base[1][4].thermal.nitout = 77
    with pytest.raises(ht.Ht3dError):
        api.ensemble_step(ctx, to_device(base), abi.MIXED)



def test_ensemble_more_members_than_one_launch_group(ctx):
    """130 members exceed one batched launch's parameter block (120 member
    records): the lockstep iteration is split into several launches per
    pseudo-iteration and stays bit-identical to per-member steps."""
    rng = np.random.default_rng(57)
    sizes = [tuple(int(v) for v in rng.integers(3, 9, size=3)) for _ in range(130)]
    base = members_np(sizes, seed=58, nitout=50)
    for *_, p in base:
        p.thermal.nitmax = p.darcy.nitmax = 500
        p.thermal.tol_rel = p.darcy.tol_rel = p.thermal.tol_abs = p.darcy.tol_abs = 1e-6
    seq, ens = to_device(base), to_device(base)
    step_sequential(ctx, seq, abi.MIXED)
    assert api.ensemble_step(ctx, ens, abi.MIXED) == [abi.OK] * len(ens)
    assert_same(ens, seq)
