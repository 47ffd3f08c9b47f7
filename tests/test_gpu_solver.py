"""GPU parity of the fused fast paths (DYREL solver, WENO5 sweep, full HRL
time step) against the oracle, FP64 and mixed precision.

Tolerances (relative, max-norm over the compared cells):
  FP64 form  : <= 1e-12 (the plain form's contract); the fused solver and the
               HRL time step round like the oracle (no FMA contraction, the
               reference's statement order, canonical tree sums) and are
               compared bit for bit where that holds
  mixed form : <= 1e-6 in T after a full step (its accuracy target), solver
               outputs within the DYREL tolerance.
Edge and corner ghost cells are excluded (the reference writes them with a
race; no consumer on the dimensionless path reads them)."""
import numpy as np
import pytest

import hydrothermal3d_gb300 as ht
from hydrothermal3d_gb300 import api, abi, hrl
from conftest import rel_err, no_edges_mask

pytestmark = pytest.mark.gpu


def rnd(rng, *s, lo=-1.0, hi=1.0):
    return np.asfortranarray(rng.uniform(lo, hi, s))


def problem(n, seed=21):
    nx, ny, nz = n
    rng = np.random.default_rng(seed)
    X = rnd(rng, nx + 2, ny + 2, nz + 2)
    R = rnd(rng, nx, ny, nz)
    k = [rnd(rng, *s, lo=0.5, hi=2.0) for s in ((nx + 1, ny, nz), (nx, ny + 1, nz), (nx, ny, nz + 1))]
    return X, R, k


BCS = {
    "thermal": ([0, 0, 1, 1, 0, 0], [0, 0, 1.0, 0.0, 0, 0]),
    "neumann": ([0] * 6, [0.0] * 6),
    "mixedbc": ([1, 0, 1, 1, 0, 1], [0.5, 0, 1.0, -1.0, 0, 2.0]),
}


@pytest.mark.parametrize("n", [(1, 1, 1), (5, 4, 3), (33, 17, 9), (40, 24, 70)])
@pytest.mark.parametrize("bc", ["thermal", "neumann", "mixedbc"])
@pytest.mark.parametrize("cX", [0.0, 25.0])
def test_fused_dyrel_fixed_iterations_fp64(ctx, orc, n, bc, cX):
    nx, ny, nz = n
    X, R, k = problem(n)
    types, vals = BCS[bc]
    prm = abi.DyrelParams.reference(nitout=10)
    dx, dy, dz = 1.0 / nx, 0.7 / ny, 1.3 / nz
    Xo, Fo, F0o = X.copy(order="F"), orc.zeros(nx, ny, nz), orc.zeros(nx, ny, nz)
    so, sto = orc.dyrel_solve_dimless(Xo, R, *k, cX, dx, dy, dz, types, vals, prm, Fo, F0o, n_iter_fixed=23)
    Xd, Fd, F0d = ht.from_numpy(X), ht.zeros(nx, ny, nz), ht.zeros(nx, ny, nz)
    std = api.dyrel_solve_dimless(ctx, Xd, ht.from_numpy(R), *[ht.from_numpy(a) for a in k], cX, dx, dy, dz, types,
                                  vals, prm, Fd, F0d, abi.FP64, n_iter_fixed=23)
    assert so == 0 and std.status == 0 and std.iters == sto.iters == 23 and std.checks == sto.checks
    m = no_edges_mask(X.shape)
    assert rel_err(ht.to_numpy(Xd), Xo, m) <= 1e-12
    # F and F0 may converge to round-off on tiny grids: compare against the
    # larger of their final size and 1e-6 of the initial residual scale
    fscale = max(np.abs(Fo).max(), np.abs(F0o).max(), 1e-6 * np.abs(R).max() * min(dx, dy, dz) ** 2)
    assert np.max(np.abs(ht.to_numpy(Fd) - Fo)) <= 1e-11 * fscale
    assert np.max(np.abs(ht.to_numpy(F0d) - F0o)) <= 1e-11 * fscale
    assert abs(std.lambda_max - sto.lambda_max) <= 1e-14 * sto.lambda_max
    assert abs(std.h1 - sto.h1) <= 1e-10
    assert abs(std.nF_abs - sto.nF_abs) <= 1e-10 * max(sto.nF_abs, 1e-6 * sto.nF_ini)


@pytest.mark.parametrize("variant", [1, 2])
@pytest.mark.parametrize("n", [(5, 4, 3), (40, 37, 33), (70, 20, 9)])
def test_fp64_solver_is_bitwise_reproducible(ctx, orc, n, variant):
    """The plain FP64 form rounds like the reference (no FMA, F/PC) and sums
    its checks in the oracle's canonical tree order: bit-identical results."""
    nx, ny, nz = n
    X, R, k = problem(n, seed=23)
    types, vals = BCS["thermal"]
    prm = abi.DyrelParams.reference(nitout=7)
    d = (1.0 / nx, 1.0 / ny, 1.0 / nz)
    Xo, Fo, F0o = X.copy(order="F"), orc.zeros(nx, ny, nz), orc.zeros(nx, ny, nz)
    so, sto = orc.dyrel_solve_dimless(Xo, R, *k, 30.0, *d, types, vals, prm, Fo, F0o, n_iter_fixed=40)
    ctx.check(ctx.lib.ht3d_ctx_set_tuning(ctx.ptr, 1, variant))
    try:
        Xd, Fd, F0d = ht.from_numpy(X), ht.zeros(nx, ny, nz), ht.zeros(nx, ny, nz)
        std = api.dyrel_solve_dimless(ctx, Xd, ht.from_numpy(R), *[ht.from_numpy(a) for a in k], 30.0, *d, types,
                                      vals, prm, Fd, F0d, abi.FP64, n_iter_fixed=40)
    finally:
        ctx.check(ctx.lib.ht3d_ctx_set_tuning(ctx.ptr, 1, 0))
    assert std.nF_abs == sto.nF_abs and std.lambda_min == sto.lambda_min and std.h1 == sto.h1
    m = no_edges_mask(X.shape)
    np.testing.assert_array_equal(ht.to_numpy(Xd)[m], Xo[m])
    np.testing.assert_array_equal(ht.to_numpy(F0d), F0o)


@pytest.mark.parametrize("n,bc,cX", [((31, 31, 31), "thermal", 200.0), ((24, 20, 28), "neumann", 0.0)])
def test_fused_dyrel_converged_solve(ctx, orc, n, bc, cX):
    """Full solve with the reference stop test: same iteration count, same solution."""
    nx, ny, nz = n
    X, R, k = problem(n, seed=22)
    if bc == "neumann":
        R -= R.mean()  # compatible right-hand side for the singular problem
    types, vals = BCS[bc]
    prm = abi.DyrelParams.reference(tol=1e-9, nitout=100, nitmax=20000)
    d = (1.0 / nx, 1.0 / ny, 1.0 / nz)
    Xo, Fo, F0o = X.copy(order="F"), orc.zeros(nx, ny, nz), orc.zeros(nx, ny, nz)
    so, sto = orc.dyrel_solve_dimless(Xo, R, *k, cX, *d, types, vals, prm, Fo, F0o)
    for prec in (abi.FP64, abi.MIXED):
        Xd, Fd, F0d = ht.from_numpy(X), ht.zeros(nx, ny, nz), ht.zeros(nx, ny, nz)
        std = api.dyrel_solve_dimless(ctx, Xd, ht.from_numpy(R), *[ht.from_numpy(a) for a in k], cX, *d, types, vals,
                                      prm, Fd, F0d, prec)
        assert std.status == 0 and std.converged == 1
        inner = (slice(1, -1),) * 3
        got, ref = ht.to_numpy(Xd)[inner], Xo[inner]
        if bc == "neumann":  # defined up to a constant
            got, ref = got - got.mean(), ref - ref.mean()
        if prec == abi.FP64:
            assert std.iters == sto.iters
            assert rel_err(got, ref) <= 1e-10
        else:
            assert abs(std.iters - sto.iters) <= prm.nitout
            assert rel_err(got, ref) <= 1e-6
            assert std.nF_rel < prm.tol_rel or std.nF_abs < prm.tol_abs


@pytest.mark.parametrize("n", [(3, 3, 3), (17, 9, 12), (64, 48, 40)])
@pytest.mark.parametrize("variant", [abi.WENO_V1, abi.WENO_V2_REF, abi.WENO_V2_FIXED])
def test_fused_weno_fp64_and_mixed(ctx, orc, n, variant):
    nx, ny, nz = n
    rng = np.random.default_rng(31)
    T = np.asfortranarray(rng.uniform(0, 1, (nx + 2, ny + 2, nz + 2)))
    V = [rnd(rng, *s) for s in ((nx + 1, ny, nz), (nx, ny + 1, nz), (nx, ny, nz + 1))]
    types, vals = [0, 0, 1, 1, 2, 2], [0, 0, 1.0, 0.0, 0, 0]
    h = (float(nx), float(ny), float(nz))
    dt = 0.2 / max(h)
    To = T.copy(order="F")
    if variant == abi.WENO_V1:
        orc.call("AdvectWithWeno5_v1", To, *V, dt, *h, orc.int6(*types), orc.dbl6(*vals), nx, ny, nz)
    else:
        import ctypes
        orc.call("AdvectWithWeno5_v2", To, *V, dt, *h, orc.int6(*types), orc.dbl6(*vals),
                 ctypes.c_int(1 if variant == abi.WENO_V2_REF else 0), nx, ny, nz)
    inner = (slice(1, -1),) * 3
    for prec, tol in ((abi.FP64, 1e-12), (abi.MIXED, 2e-6)):
        Td = ht.from_numpy(T)
        api.weno5_advect(ctx, Td, *[ht.from_numpy(v) for v in V], dt, *h, types, vals, variant, prec)
        got = ht.to_numpy(Td)
        assert rel_err(got[inner], To[inner]) <= tol
        np.testing.assert_array_equal(got[0], T[0])  # ghosts untouched


def _vel_err(Vd, V):
    """Max-norm difference of the three face velocities relative to max|V|."""
    scale = max(np.abs(v).max() for v in V)
    return max(np.max(np.abs(ht.to_numpy(a) - b)) for a, b in zip(Vd, V)) / scale


def _hrl_fp64_vs_oracle(ctx, orc, n, steps, nitout):
    nx, ny, nz = n
    T, P, ktv, kfv = hrl.initial_fields(nx, ny, nz, seed=1)
    p_o = hrl.params(nx, ny, nz, nitout=nitout)
    p_d = hrl.params(nx, ny, nz, nitout=nitout)
    V = [np.zeros(s, order="F") for s in ((nx + 1, ny, nz), (nx, ny + 1, nz), (nx, ny, nz + 1))]
    Td, Pd = ht.from_numpy(T), ht.from_numpy(P)
    Vd = [ht.zeros(*v.shape) for v in V]
    ktd, kfd = ht.from_numpy(ktv), ht.from_numpy(kfv)
    m = no_edges_mask(T.shape)
    inner = (slice(1, -1),) * 3
    for step in range(steps):
        s, st_t, st_d = orc.step_hrl(T, P, ktv, kfv, *V, p_o)
        assert s == 0
        gt, gd = api.step_hrl(ctx, Td, Pd, ktd, kfd, *Vd, p_d, abi.FP64)
        assert (gt.iters, gd.iters) == (st_t.iters, st_d.iters), step
        np.testing.assert_array_equal(ht.to_numpy(Td)[m], T[m])
        Pn, Pg = P[inner], ht.to_numpy(Pd)[inner]
        np.testing.assert_array_equal(Pg, Pn)
        assert rel_err(Pg - Pg.mean(), Pn - Pn.mean()) <= 1e-12
        assert _vel_err(Vd, V) <= 1e-12, step
        assert abs(p_d.dt - p_o.dt) <= 1e-12 * p_o.dt


@pytest.mark.parametrize("n", [(16, 16, 16), (33, 31, 29)])
def test_step_hrl_fp64_matches_oracle(ctx, orc, n):
    """Three HRL time steps: same iteration counts, T and P bit for bit, the
    Darcy velocities within 1e-12 of max|V|, the same adapted dt."""
    _hrl_fp64_vs_oracle(ctx, orc, n, 3, 100)


def test_hrl_63_ten_steps_match_oracle(ctx, orc):
    """The 63^3 workload as stated (Ra 1000, tolerance 1e-8, nitout 1000, WENO5
    v1, adaptive dt, 10 time steps) against the oracle on the host: T and P
    bit for bit after every step."""
    _hrl_fp64_vs_oracle(ctx, orc, (63, 63, 63), 10, 1000)


def test_step_hrl_mixed_error_vs_oracle(ctx, orc):
    nx = ny = nz = 32
    T, P, ktv, kfv = hrl.initial_fields(nx, ny, nz, seed=1)
    p_o = hrl.params(nx, ny, nz, nitout=100)
    p_d = hrl.params(nx, ny, nz, nitout=100)
    V = [np.zeros(s, order="F") for s in ((nx + 1, ny, nz), (nx, ny + 1, nz), (nx, ny, nz + 1))]
    Td, Pd = ht.from_numpy(T), ht.from_numpy(P)
    Vd = [ht.zeros(*v.shape) for v in V]
    ktd, kfd = ht.from_numpy(ktv), ht.from_numpy(kfv)
    inner = (slice(1, -1),) * 3
    for step in range(3):
        orc.step_hrl(T, P, ktv, kfv, *V, p_o)
        gt, gd = api.step_hrl(ctx, Td, Pd, ktd, kfd, *Vd, p_d, abi.MIXED)
        assert gt.status == 0 and gd.status == 0
        # the same dt sequence keeps the comparison meaningful
        p_d.dt = p_o.dt
    assert rel_err(ht.to_numpy(Td)[inner], T[inner]) <= 1e-6


@pytest.mark.parametrize("n", [(1, 1, 1), (3, 2, 2), (4, 5, 3), (31, 7, 5), (36, 5, 4), (127, 3, 2), (129, 6, 3)])
@pytest.mark.parametrize("bc", ["thermal", "mixedbc"])
@pytest.mark.parametrize("niter", [40, 32, 37])
def test_mixed_fixed_iterations_track_fp64(ctx, orc, n, bc, niter):
    """The mixed form's padded FP32 inner kernel (4 cells per thread, warp
    shuffles across quads, scalar loads at warp and row edges) follows the
    FP64 iteration: the update X - X0 after 32-40 pseudo-iterations matches the
    oracle's to FP32 accuracy, and the face ghosts hold the BC of the state
    before the last iteration like the reference's.  Sizes cover nx < 4,
    nx % 4 == 0, rows that end inside a warp, nx + 1 = 128 and rows longer
    than one warp; the last iteration is a check (40), an FP64 refresh (32)
    or an FP32 inner iteration (37)."""
    nx, ny, nz = n
    X, R, k = problem(n, seed=31)
    types, vals = BCS[bc]
    prm = abi.DyrelParams.reference(nitout=10)
    d = (1.0 / nx, 0.8 / ny, 1.1 / nz)
    Xo, Fo, F0o = X.copy(order="F"), orc.zeros(nx, ny, nz), orc.zeros(nx, ny, nz)
    so, sto = orc.dyrel_solve_dimless(Xo, R, *k, 40.0, *d, types, vals, prm, Fo, F0o, n_iter_fixed=niter)
    ctx.set_tuning(abi.TUNE_MIXED_REFRESH, 8)
    ctx.set_tuning(abi.TUNE_TIME_INNER, 1)
    ctx.inner_timing(reset=True)
    try:
        Xd, Fd, F0d = ht.from_numpy(X), ht.zeros(nx, ny, nz), ht.zeros(nx, ny, nz)
        std = api.dyrel_solve_dimless(ctx, Xd, ht.from_numpy(R), *[ht.from_numpy(a) for a in k], 40.0, *d, types,
                                      vals, prm, Fd, F0d, abi.MIXED, n_iter_fixed=niter)
        ms, launches = ctx.inner_timing(reset=True)
    finally:
        ctx.set_tuning(abi.TUNE_MIXED_REFRESH, 512)
        ctx.set_tuning(abi.TUNE_TIME_INNER, 0)
    assert so == 0 and std.status == 0 and std.iters == niter and std.checks == sto.checks
    # checks at 1, 2 and every 10th iteration, FP64 refreshes at every other 8th
    fp64_iters = [it for it in range(1, niter + 1) if it <= 2 or it % 10 == 0 or it % 8 == 0]
    assert launches == niter - len(fp64_iters) and ms > 0.0
    m = no_edges_mask(X.shape)
    inner = (slice(1, -1),) * 3
    du_ref, du = (Xo - X)[inner], (ht.to_numpy(Xd) - X)[inner]
    assert rel_err(du, du_ref) <= 1e-4
    assert rel_err(ht.to_numpy(Xd), Xo, m) <= 1e-6
    # F and F0 shrink as the iteration converges (to ~1e-7 on one cell):
    # compare against the larger of their final size and 1e-3 of the first
    # iteration's scale R*dx^2
    fscale = max(np.abs(Fo).max(), np.abs(F0o).max(), 1e-3 * np.abs(R).max() * min(d) ** 2)
    assert np.max(np.abs(ht.to_numpy(F0d) - F0o)) <= 1e-4 * fscale
    assert np.max(np.abs(ht.to_numpy(Fd) - Fo)) <= 1e-3 * fscale


@pytest.mark.parametrize("n", [(1, 1, 1), (2, 3, 2), (5, 4, 3), (30, 14, 9), (31, 15, 40), (64, 29, 33), (95, 47, 70),
                               (128, 15, 4), (129, 15, 3), (130, 29, 6), (255, 16, 3), (257, 17, 3)])
@pytest.mark.parametrize("niter,refresh", [(40, 8), (37, 8), (25, 256), (100, 16)])
@pytest.mark.parametrize("zchunk", [2, 7, 64])
def test_mixed_temporal_blocking_is_bit_identical(ctx, n, niter, refresh, zchunk):
    """k_mixed_inner2 (two iterations per pass through memory, with halo
    recomputation across tiles and z-chunks) gives bit for bit the result of
    one k_mixed_inner launch per iteration: X, F, F0 and the check sums.
    Sizes cover one to three tiles of 128 cells in x (and a last tile of one
    cell) and of 14 rows in y."""
    nx, ny, nz = n
    X, R, k = problem(n, seed=37)
    types, vals = BCS["mixedbc"]
    prm = abi.DyrelParams.reference(nitout=10)
    d = (1.0 / nx, 0.9 / ny, 1.2 / nz)
    out = []
    ctx.set_tuning(abi.TUNE_MIXED_REFRESH, refresh)
    try:
        for temporal in (0, zchunk):
            ctx.set_tuning(abi.TUNE_TEMPORAL, temporal)
            Xd, Fd, F0d = ht.from_numpy(X), ht.zeros(nx, ny, nz), ht.zeros(nx, ny, nz)
            st = api.dyrel_solve_dimless(ctx, Xd, ht.from_numpy(R), *[ht.from_numpy(a) for a in k], 30.0, *d, types,
                                         vals, prm, Fd, F0d, abi.MIXED, n_iter_fixed=niter)
            out.append((ht.to_numpy(Xd), ht.to_numpy(Fd), ht.to_numpy(F0d), st.nF_abs, st.lambda_min, st.iters))
    finally:
        ctx.set_tuning(abi.TUNE_TEMPORAL, 1)
        ctx.set_tuning(abi.TUNE_MIXED_REFRESH, 512)
    a, b = out
    m = no_edges_mask(X.shape)
    np.testing.assert_array_equal(a[0][m], b[0][m])
    np.testing.assert_array_equal(a[1], b[1])
    np.testing.assert_array_equal(a[2], b[2])
    assert a[3:] == b[3:]


def test_bounded_wait_runs_out_and_context_recovers(ctx):
    """HT3D_TUNE_WAIT_TEST: the first two-iteration pass never issues the copies
    of plane 1, its bounded mbarrier wait gives up, the CTA waits for the copies
    it did issue and returns, and the solve reports HT3D_ERR_TIMEOUT.  The same
    context then solves normally: bit-identical to the per-iteration kernel."""
    n = (30, 14, 9)
    nx, ny, nz = n
    X, R, k = problem(n, seed=43)
    types, vals = BCS["mixedbc"]
    prm = abi.DyrelParams.reference(nitout=10)
    d = (1.0 / nx, 0.9 / ny, 1.2 / nz)

    def solve():
        Xd, Fd, F0d = ht.from_numpy(X), ht.zeros(nx, ny, nz), ht.zeros(nx, ny, nz)
        api.dyrel_solve_dimless(ctx, Xd, ht.from_numpy(R), *[ht.from_numpy(a) for a in k], 30.0, *d, types, vals,
                                prm, Fd, F0d, abi.MIXED, n_iter_fixed=9)
        return ht.to_numpy(Xd), ht.to_numpy(Fd), ht.to_numpy(F0d)

    try:
        ctx.set_tuning(abi.TUNE_TEMPORAL, 3)
        ctx.set_tuning(abi.TUNE_WAIT_TEST, 2)
        with pytest.raises(api.Ht3dError) as e:
            solve()
        assert e.value.status == abi.ERR_TIMEOUT
        paired = solve()  # the hook is spent: a normal solve on the same context
        ctx.set_tuning(abi.TUNE_TEMPORAL, 0)
        single = solve()
    finally:
        ctx.set_tuning(abi.TUNE_WAIT_TEST, 0)
        ctx.set_tuning(abi.TUNE_TEMPORAL, 1)
    m = no_edges_mask(X.shape)
    np.testing.assert_array_equal(paired[0][m], single[0][m])
    np.testing.assert_array_equal(paired[1], single[1])
    np.testing.assert_array_equal(paired[2], single[2])
