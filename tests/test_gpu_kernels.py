"""GPU parity of the granular, reference-shaped kernels against the oracle.

These translation units are compiled with -fmad=false, so with the same
statement order the results agree with the oracle to the last bit or so; the
tolerance written here is 1e-15 relative (max-norm)."""
import ctypes

import numpy as np
import pytest
import torch

import hydrothermal3d_gb300 as ht
from hydrothermal3d_gb300 import api, abi
from conftest import rel_err

pytestmark = pytest.mark.gpu
TOL = 1e-15
SIZES = [(1, 1, 1), (2, 3, 1), (5, 4, 3), (33, 17, 9)]


def rnd(rng, *s, lo=-1.0, hi=1.0):
    return np.asfortranarray(rng.uniform(lo, hi, s))


def dev(a):
    return ht.from_numpy(a)


def host(t):
    return ht.to_numpy(t)


@pytest.mark.parametrize("n", SIZES)
def test_compute_flux_and_residuals(ctx, orc, n):
    nx, ny, nz = n
    rng = np.random.default_rng(11)
    A, kx, ky, kz = rnd(rng, nx + 2, ny + 2, nz + 2), rnd(rng, nx + 1, ny, nz, lo=.5), rnd(rng, nx, ny + 1, nz, lo=.5), rnd(rng, nx, ny, nz + 1, lo=.5)
    R = rnd(rng, nx, ny, nz)
    h = (1.3, 0.7, 2.1)
    q = [np.zeros(s, order="F") for s in ((nx + 1, ny, nz), (nx, ny + 1, nz), (nx, ny, nz + 1))]
    orc.call("ComputeFlux", *q, kx, ky, kz, A, *h, nx, ny, nz)
    qd = [ht.zeros(*s.shape) for s in q]
    api.ComputeFlux(ctx, *qd, dev(kx), dev(ky), dev(kz), dev(A), *h)
    for a, b in zip(qd, q):
        assert rel_err(host(a), b) <= TOL
    # residuals and UpdateT!
    F = np.zeros((nx, ny, nz), order="F")
    Fd = ht.zeros(nx, ny, nz)
    orc.call("ResidualDiffusion", F, R, *q, *h, nx, ny, nz)
    api.ResidualDiffusion(ctx, Fd, dev(R), *[dev(x) for x in q], *h)
    assert rel_err(host(Fd), F) <= TOL
    orc.call("ResidualDiffusionTransient", F, A, R, *q, 4.5, *h, nx, ny, nz)
    api.ResidualDiffusionTransient(ctx, Fd, dev(A), dev(R), *[dev(x) for x in q], 4.5, *h)
    assert rel_err(host(Fd), F) <= TOL
    T = A.copy(order="F")
    Td = dev(T)
    orc.call("UpdateT", F, T, R, *q, 4.5, 0.01, *h, nx, ny, nz)
    api.UpdateT(ctx, Fd, Td, dev(R), *[dev(x) for x in q], 4.5, 0.01, *h)
    assert rel_err(host(Fd), F) <= TOL and rel_err(host(Td), T) <= TOL


@pytest.mark.parametrize("n", SIZES)
def test_updates_and_init(ctx, orc, n):
    nx, ny, nz = n
    rng = np.random.default_rng(12)
    F, F0, X = rnd(rng, nx, ny, nz), rnd(rng, nx, ny, nz), rnd(rng, nx + 2, ny + 2, nz + 2)
    for name, args in (("UpdateP", (0.9, 0.05)), ("DYRELUpdate", (0.95, 0.3, 0.05))):
        F0o, Xo = F0.copy(order="F"), X.copy(order="F")
        F0d, Xd = dev(F0), dev(X)
        orc.call(name, F0o, Xo, F, *args, nx, ny, nz)
        getattr(api, name)(ctx, F0d, Xd, dev(F), *args)
        assert rel_err(host(F0d), F0o) <= TOL and rel_err(host(Xd), Xo) <= TOL
    T, kv = rnd(rng, nx + 2, ny + 2, nz + 2), rnd(rng, nx + 1, ny + 1, nz + 1, lo=.5)
    shp = ((nx, ny + 1, nz), (nx + 1, ny, nz), (nx, ny + 1, nz), (nx, ny, nz + 1))
    o = [np.zeros(s, order="F") for s in shp]
    d = [ht.zeros(*s) for s in shp]
    orc.call("InitDarcy", *o, T, kv, 1.0, nx, ny, nz)
    api.InitDarcy(ctx, *d, dev(T), dev(kv), 1.0)
    for a, b in zip(d, o):
        assert rel_err(host(a), b) <= TOL
    Rt, Rtd = np.zeros((nx, ny, nz), order="F"), ht.zeros(nx, ny, nz)
    orc.call("InitThermal_dimless", Rt, *o[1:], T, kv, 3.0, nx, ny, nz)
    api.InitThermal(ctx, Rtd, *d[1:], dev(T), dev(kv), 3.0)
    assert rel_err(host(Rtd), Rt) <= TOL
    Rp, Rpd = np.zeros((nx, ny, nz), order="F"), ht.zeros(nx, ny, nz)
    orc.call("Compute_Rp", Rp, o[2], o[0], 77.0, 3.0, nx, ny, nz)
    api.Compute_Rp(ctx, Rpd, d[2], d[0], 77.0, 3.0)
    assert rel_err(host(Rpd), Rp) <= TOL
    orc.call("KillNorthSouthFluxes", o[0], nx, ny, nz)
    api.KillNorthSouthFluxes(ctx, d[0])
    assert np.array_equal(host(d[0]), o[0])
    P = rnd(rng, nx + 2, ny + 2, nz + 2)
    V = [np.zeros(s, order="F") for s in ((nx + 1, ny, nz), (nx, ny + 1, nz), (nx, ny, nz + 1))]
    Vd = [ht.zeros(*v.shape) for v in V]
    orc.call("Init_vel", *V, *o[1:], P, o[0], 50.0, 1.5, 2.5, 3.5, nx, ny, nz)
    api.Init_vel(ctx, *Vd, *d[1:], dev(P), d[0], 50.0, 1.5, 2.5, 3.5)
    for a, b in zip(Vd, V):
        assert rel_err(host(a), b) <= TOL


@pytest.mark.parametrize("n", SIZES)
def test_face_bcs_including_edges(ctx, orc, n):
    nx, ny, nz = n
    rng = np.random.default_rng(13)
    X = rnd(rng, nx + 2, ny + 2, nz + 2)
    for types, vals in (([0, 0, 1, 1, 0, 0], [0, 0, 1.0, 0.0, 0, 0]), ([1, 1, 0, 1, 1, 0], [.3, .4, 0, -2, 5, 0])):
        Xo = X.copy(order="F")
        Xd = dev(X)
        orc.call("SetFaceBCs", Xo, orc.int6(*types), orc.dbl6(*vals), nx, ny, nz)
        api.SetFaceBCs(ctx, Xd, types, vals)
        np.testing.assert_array_equal(host(Xd), Xo)  # snapshot semantics, edges and corners included
    Xo = X.copy(order="F")
    Xd = dev(X)
    orc.call("SetFaceBCs", Xo, orc.int6(0, 0, 1, 1, 0, 0), orc.dbl6(0, 0, 0.25, 0.0, 0, 0), nx, ny, nz)
    api.SetPressureBCs(ctx, Xd, 0.25, 0.0)
    np.testing.assert_array_equal(host(Xd), Xo)


@pytest.mark.parametrize("n", SIZES)
def test_gershgorin_swap_rayleigh_copies(ctx, orc, n):
    nx, ny, nz = n
    rng = np.random.default_rng(14)
    kx, ky, kz = rnd(rng, nx + 1, ny, nz, lo=.5), rnd(rng, nx, ny + 1, nz, lo=.5), rnd(rng, nx, ny, nz + 1, lo=.5)
    rC = rnd(rng, nx, ny, nz, lo=.5)
    G, D = np.zeros((nx, ny, nz), order="F"), np.zeros((nx, ny, nz), order="F")
    Gd, Dd = ht.zeros(nx, ny, nz), ht.zeros(nx, ny, nz)
    orc.call("GershgorinPoisson", G, D, rC, kx, ky, kz, 1.0, 0.1, 0.2, 0.3, 0.4, nx, ny, nz)
    api.GershgorinPoisson(ctx, Gd, Dd, dev(rC), dev(kx), dev(ky), dev(kz), 1.0, 0.1, 0.2, 0.3, 0.4)
    assert rel_err(host(Gd), G) <= TOL and rel_err(host(Dd), D) <= TOL
    orc.call("GershgorinHydro", G, rC, kx, ky, kz, 1.0, 0.1, 0.2, 0.3, 0.4, nx, ny, nz)
    api.GershgorinHydro(ctx, Gd, dev(rC), dev(kx), dev(ky), dev(kz), 1.0, 0.1, 0.2, 0.3, 0.4)
    assert rel_err(host(Gd), G) <= TOL
    X0, Y0 = rnd(rng, nx + 2, ny + 2, nz + 2), rnd(rng, nx, ny, nz)
    Xc, Yc = np.zeros((nx, ny, nz), order="F"), np.zeros((nx, ny, nz), order="F")
    Xcd, Ycd = ht.zeros(nx, ny, nz), ht.zeros(nx, ny, nz)
    orc.call("SwapDYREL", Xc, Yc, X0, Y0, nx, ny, nz)
    api.SwapDYREL(ctx, Xcd, Ycd, dev(X0), dev(Y0))
    assert np.array_equal(host(Xcd), Xc) and np.array_equal(host(Ycd), Yc)
    a, b, c = rnd(rng, nx, ny, nz), rnd(rng, nx, ny, nz), rnd(rng, nx, ny, nz)
    orc.call("RayleighQuotientNumerator", G, a, b, c, 0.37, a.size)
    api.RayleighQuotientNumerator(ctx, Gd, dev(a), dev(b), dev(c), 0.37)
    assert rel_err(host(Gd), G) <= TOL
    orc.call("RayleighQuotientDenominator", G, a, 0.37, a.size)
    api.RayleighQuotientDenominator(ctx, Gd, dev(a), 0.37)
    assert rel_err(host(Gd), G) <= TOL
    orc.call("Multiply", G, a, b, a.size)
    api.Multiply(ctx, Gd, dev(a), dev(b))
    assert np.array_equal(host(Gd), G)
    Ad = dev(a)
    api.Cpy_all_to_inn(ctx, dev(X0), Ad)
    api.ResetA(ctx, Ad, Gd)
    assert float(Ad.abs().max()) == 0.0 and float(Gd.abs().max()) == 0.0


@pytest.mark.parametrize("n", [(1, 1, 1), (37, 5, 3), (64, 64, 64)])
def test_reductions(ctx, orc, n):
    rng = np.random.default_rng(15)
    a = rnd(rng, *n)
    ad = dev(a)
    assert abs(api.sum_g(ctx, ad) - a.sum()) <= 1e-12 * np.abs(a).sum()
    assert api.maximum_g(ctx, ad) == a.max() and api.minimum_g(ctx, ad) == a.min()
    assert abs(api.mean_abs_g(ctx, ad) - np.abs(a).mean()) <= 1e-13 * np.abs(a).mean()
    assert api.maximum_abs_g(ctx, ad) == np.abs(a).max()
    # deterministic: same answer twice
    assert api.sum_g(ctx, ad) == api.sum_g(ctx, ad)


@pytest.mark.parametrize("n", [(3, 3, 3), (7, 5, 4), (33, 9, 17)])
def test_weno_granular_v1_and_v2(ctx, orc, n):
    nx, ny, nz = n
    rng = np.random.default_rng(16)
    T = rnd(rng, nx + 2, ny + 2, nz + 2)
    Tc = np.asfortranarray(T[1:-1, 1:-1, 1:-1])
    h = (2.0, 3.0, 5.0)
    for axis in range(3):
        for ghosted, src in ((0, Tc), (1, T)):
            for tL, tR in ((0, 1), (2, 2), (1, 0)):
                X = np.zeros((nx + 6, ny + 6, nz + 6), order="F")
                Xd = ht.zeros(nx + 6, ny + 6, nz + 6)
                orc.call("Boundaries_Weno5", X, src, ctypes.c_int(axis), ctypes.c_int(tL), 0.7, ctypes.c_int(tR), -0.2,
                         ctypes.c_int(ghosted), nx, ny, nz)
                api.Boundaries_Weno5(ctx, Xd, dev(src), axis, tL, 0.7, tR, -0.2)
                np.testing.assert_array_equal(host(Xd), X)
        for sign in (-1, 1):
            v = [np.zeros((nx, ny, nz), order="F") for _ in range(5)]
            vd = [ht.zeros(nx, ny, nz) for _ in range(5)]
            orc.call("Gradients_Weno5", *v, X, ctypes.c_int(axis), ctypes.c_int(sign), *h, nx, ny, nz)
            api.Gradients_Weno5(ctx, *vd, Xd, axis, sign, *h)
            for a, b in zip(vd, v):
                assert np.array_equal(host(a), b)
            dF, dFd = np.zeros((nx, ny, nz), order="F"), ht.zeros(nx, ny, nz)
            orc.call("dFdx_Weno5", dF, *v, dF.size)
            api.dFdx_Weno5(ctx, dFd, *vd)
            assert rel_err(host(dFd), dF) <= 1e-14
        shape = [nx, ny, nz]
        shape[axis] += 1
        V = rnd(rng, *shape)
        V.flat[::7] = 0.0
        # faces the comparisons V < 0 / V > 0 both reject (-0, NaN) or take (+-inf)
        # leave / set the outputs; the outputs start at a sentinel so a skipped write shows
        V.flat[3::11] = -0.0
        V.flat[5::13] = np.nan
        V.flat[2::17] = np.inf
        V.flat[4::19] = -np.inf
        Vm, Vp = np.full((nx, ny, nz), 7.0, order="F"), np.full((nx, ny, nz), 7.0, order="F")
        Vmd, Vpd = dev(Vm), dev(Vp)
        orc.call("VPlusMinus", Vm, Vp, V, ctypes.c_int(axis), nx, ny, nz)
        api.VPlusMinus(ctx, Vmd, Vpd, dev(V), axis)
        assert np.array_equal(host(Vmd), Vm) and np.array_equal(host(Vpd), Vp)
        V[~np.isfinite(V)] = 0.5  # the advection below wants finite velocities
        for quirk in (0, 1):
            To, Td = T.copy(order="F"), dev(T)
            orc.call("Advect_v2", To, X, V, ctypes.c_int(axis), 0.01, *h, ctypes.c_int(quirk), nx, ny, nz)
            api.Advect_v2(ctx, Td, Xd, dev(V), axis, 0.01, *h, quirk=quirk)
            assert rel_err(host(Td), To) <= 1e-14


@pytest.mark.parametrize("n", [(4, 3, 5), (33, 17, 9)])
def test_weno_v1_pieces_and_copies(ctx, orc, n):
    """Advect! / TimeAveraging! (v1 and v2), Cpy_inn_to_all!, ArrayEqualArray!."""
    nx, ny, nz = n
    N = nx * ny * nz
    rng = np.random.default_rng(71)
    F, Vp, dm, Vm, dp = (rnd(rng, nx, ny, nz) for _ in range(5))
    Fo, Fd = F.copy(order="F"), dev(F)
    orc.call("Advect_v1", Fo, Vp, dm, Vm, dp, 0.013, N)
    api.Advect_v1(ctx, Fd, dev(Vp), dev(dm), dev(Vm), dev(dp), 0.013)
    assert rel_err(host(Fd), Fo) <= TOL
    Fold = rnd(rng, nx, ny, nz)
    for order in (1.0, 2.0, 3.0):  # 1/3 is inexact: the weights the host forms must match per-cell ones
        Fo, Fd = F.copy(order="F"), dev(F)
        orc.call("TimeAveraging_v1", Fo, Fold, order, N)
        api.TimeAveraging_v1(ctx, Fd, dev(Fold), order)
        assert rel_err(host(Fd), Fo) <= TOL
        Fex = rnd(rng, nx + 2, ny + 2, nz + 2)
        Fo, Fd = Fex.copy(order="F"), dev(Fex)
        orc.call("TimeAveraging_v2", Fo, Fold, order, nx, ny, nz)
        api.TimeAveraging_v2(ctx, Fd, dev(Fold), order)
        assert rel_err(host(Fd), Fo) <= TOL
    Bex = rnd(rng, nx + 2, ny + 2, nz + 2)
    A, Ad = np.zeros((nx, ny, nz), order="F"), ht.zeros(nx, ny, nz)
    orc.call("Cpy_inn_to_all", A, Bex, nx, ny, nz)
    api.Cpy_inn_to_all(ctx, Ad, dev(Bex))
    assert np.array_equal(host(Ad), A) and np.array_equal(A, Bex[1:-1, 1:-1, 1:-1])
    C, Cd = np.zeros((nx, ny, nz), order="F"), ht.zeros(nx, ny, nz)
    orc.call("ArrayEqualArray", C, F, N)
    api.ArrayEqualArray(ctx, Cd, dev(F))
    assert np.array_equal(host(Cd), C) and np.array_equal(C, F)


def test_dyrel_iterate_f32_tracks_fp64(ctx):
    """The FP32 iteration on the reference layout (ht3d_dyrel_iterate_f32,
    1/PC) follows the FP64 one (ht3d_dyrel_iterate, PC) to FP32 accuracy."""
    nx, ny, nz = 19, 11, 7
    rng = np.random.default_rng(73)
    X = rnd(rng, nx + 2, ny + 2, nz + 2)
    R = rnd(rng, nx, ny, nz)
    k = [rnd(rng, *s, lo=0.5, hi=2.0) for s in ((nx + 1, ny, nz), (nx, ny + 1, nz), (nx, ny, nz + 1))]
    PC = rnd(rng, nx, ny, nz, lo=600.0, hi=900.0)
    bt, bv = abi.int6(0, 0, 1, 1, 0, 0), abi.dbl6(0, 0, 1.0, 0.0, 0, 0)
    d = (1 / nx, 1 / ny, 1 / nz)
    out = {}
    for prec in ("f64", "f32"):
        t = torch.float64 if prec == "f64" else torch.float32
        Xd = dev(X).to(t).permute(2, 1, 0).contiguous().permute(2, 1, 0)
        Rd, F0 = dev(R).to(t), ht.zeros(nx, ny, nz, dtype=t)
        kd = [dev(a).to(t) for a in k]
        Pd = dev(PC).to(t) if prec == "f64" else (1.0 / dev(PC)).to(t)
        fields = [a.permute(2, 1, 0).contiguous().permute(2, 1, 0) for a in (Rd, *kd, Pd)]
        name = "ht3d_dyrel_iterate" if prec == "f64" else "ht3d_dyrel_iterate_f32"
        ctx.call(name, Xd.data_ptr(), *[a.data_ptr() for a in fields], F0.data_ptr(), 25.0, *d, bt, bv, 0.9, 0.05,
                 0.0008, 30, nx, ny, nz)
        out[prec] = Xd.double().cpu().numpy()
    inner = (slice(1, -1),) * 3
    du64, du32 = (out["f64"] - X)[inner], (out["f32"] - X)[inner]
    assert rel_err(du32, du64) <= 1e-4


def test_ctx_stream_and_sync_controls(ctx):
    """ht3d_ctx_set_sync / _set_stream / _synchronize and the last-error text."""
    lib = ctx.lib
    s = torch.cuda.Stream()
    assert lib.ht3d_ctx_set_stream(ctx.ptr, s.cuda_stream) == abi.OK
    assert lib.ht3d_ctx_set_sync(ctx.ptr, 0) == abi.OK
    a = ht.zeros(8, 8, 8) + 1.0
    b = ht.zeros(8, 8, 8)
    torch.cuda.synchronize()
    with torch.cuda.stream(s):
        api.ArrayEqualArray(ctx, b, a)
    assert lib.ht3d_ctx_synchronize(ctx.ptr) == abi.OK
    assert float(b.min()) == 1.0
    assert lib.ht3d_ctx_set_sync(ctx.ptr, 1) == abi.OK
    assert lib.ht3d_ctx_set_stream(ctx.ptr, None) == abi.OK  # a private stream of its own
    assert lib.ht3d_ctx_synchronize(ctx.ptr) == abi.OK
    assert lib.ht3d_ctx_set_stream(ctx.ptr, ctx.stream) == abi.OK  # back to the tests' stream
    # rejected calls (checked on the host before any launch) leave a readable
    # message and an unchanged, usable context
    p = a.data_ptr()
    st = lib.ht3d_ComputeFlux(ctx.ptr, p, p, p, p, p, p, p, 1.0, 1.0, 1.0, 0, 4, 4)  # zero cells
    assert st == abi.ERR_ARG and len(lib.ht3d_ctx_last_error(ctx.ptr)) > 0
    st = lib.ht3d_ComputeFlux(ctx.ptr, None, None, None, None, None, None, None, 1.0, 1.0, 1.0, 4, 4, 4)
    assert st == abi.ERR_ARG and b"null" in lib.ht3d_ctx_last_error(ctx.ptr)
    api.ArrayEqualArray(ctx, b, a)
