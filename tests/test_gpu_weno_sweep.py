"""Standalone WENO5 sweep: FP32 (ht3d_weno5_advect_f32), mixed and FP64
fused sweeps against the oracle's AdvectWithWeno5 on a blob advected by a
discretely divergence-free velocity.

Tolerances (max-norm, relative to max |T|): FP64 1e-12, mixed 2e-6,
FP32 storage and arithmetic 2e-5 per sweep."""
import ctypes

import numpy as np
import pytest
import torch

import hydrothermal3d_gb300 as ht
from hydrothermal3d_gb300 import api, abi, sweep
from conftest import rel_err

pytestmark = pytest.mark.gpu

BCS = {
    "hrl": ([0, 0, 1, 1, 0, 0], [0, 0, 1.0, 0.0, 0, 0]),
    "periodic": ([2, 2, 0, 0, 2, 2], [0.0] * 6),
}


def oracle_sweep(orc, T, V, dt, h, types, vals, variant):
    nx, ny, nz = (s - 2 for s in T.shape)
    To = T.copy(order="F")
    if variant == abi.WENO_V1:
        orc.call("AdvectWithWeno5_v1", To, *V, dt, *h, orc.int6(*types), orc.dbl6(*vals), nx, ny, nz)
    else:
        orc.call("AdvectWithWeno5_v2", To, *V, dt, *h, orc.int6(*types), orc.dbl6(*vals),
                 ctypes.c_int(1 if variant == abi.WENO_V2_REF else 0), nx, ny, nz)
    return To


@pytest.mark.parametrize("n", [(24, 20, 28), (33, 17, 9), (3, 5, 4)])
@pytest.mark.parametrize("variant", [abi.WENO_V1, abi.WENO_V2_REF, abi.WENO_V2_FIXED])
@pytest.mark.parametrize("bc", ["hrl", "periodic"])
def test_sweep_precisions_against_oracle(ctx, orc, n, variant, bc):
    nx, ny, nz = n
    Vd = sweep.curl_velocity(nx, ny, nz, seed=6)
    Td = sweep.blob(nx, ny, nz)
    T, V = ht.to_numpy(Td), [ht.to_numpy(v) for v in Vd]
    types, vals = BCS[bc]
    h = (float(nx), float(ny), float(nz))
    dt = sweep.cfl_dt(nx, ny, nz, cfl=0.5)
    # two sweeps, so the second one starts from an advected field
    To = oracle_sweep(orc, oracle_sweep(orc, T, V, dt, h, types, vals, variant), V, dt, h, types, vals, variant)
    inner = (slice(1, -1),) * 3
    for prec, tol in ((abi.FP64, 1e-12), (abi.MIXED, 2e-6)):
        Tg = ht.from_numpy(T)
        for _ in range(2):
            api.weno5_advect(ctx, Tg, *Vd, dt, *h, types, vals, variant, prec)
        assert rel_err(ht.to_numpy(Tg)[inner], To[inner]) <= tol, prec
    T32 = Td.float().permute(2, 1, 0).contiguous().permute(2, 1, 0)
    V32 = [v.float().permute(2, 1, 0).contiguous().permute(2, 1, 0) for v in Vd]
    for _ in range(2):
        api.weno5_advect_f32(ctx, T32, *V32, dt, *h, types, vals, variant)
    got = T32.double().cpu().numpy()
    assert rel_err(got[inner], To[inner]) <= 2e-5
    np.testing.assert_array_equal(got[0], np.float32(T[0]))  # ghosts untouched


@pytest.mark.parametrize("n", [(65, 66, 130), (97, 49, 96), (255, 8, 7)])
@pytest.mark.parametrize("variant", [abi.WENO_V1, abi.WENO_V2_REF])
def test_sweep_f32_segments_against_oracle(ctx, orc, n, variant):
    """The FP32 march kernels split lines into segments (x: several lanes of a
    warp per shared-memory row; y, z: several threads per line): sizes whose
    segments end one or two cells before the line's end, or right at it."""
    nx, ny, nz = n
    Vd = sweep.curl_velocity(nx, ny, nz, seed=6)
    Td = sweep.blob(nx, ny, nz)
    T, V = ht.to_numpy(Td), [ht.to_numpy(v) for v in Vd]
    types, vals = BCS["hrl"]
    h = (float(nx), float(ny), float(nz))
    dt = sweep.cfl_dt(nx, ny, nz, cfl=0.5)
    To = oracle_sweep(orc, T, V, dt, h, types, vals, variant)
    inner = (slice(1, -1),) * 3
    T32 = Td.float().permute(2, 1, 0).contiguous().permute(2, 1, 0)
    V32 = [v.float().permute(2, 1, 0).contiguous().permute(2, 1, 0) for v in Vd]
    api.weno5_advect_f32(ctx, T32, *V32, dt, *h, types, vals, variant)
    got = T32.double().cpu().numpy()
    assert rel_err(got[inner], To[inner]) <= 2e-5


@pytest.mark.parametrize("n", [(511, 40, 36), (383, 24, 20), (36, 383, 24), (24, 20, 383)])
def test_sweep_f32_long_lines_track_fp64(ctx, n):
    """One FP32 sweep on boxes long along one axis (many segments per line,
    flow along every axis) within 1e-6 of the FP64 sweep: the FP32 rounding of
    a sweep is ~1e-7 there, so any cell computed from a stale neighbour (a
    segment seam read while another block updates it) shows up."""
    nx, ny, nz = n
    V = sweep.curl_velocity(nx, ny, nz, seed=6)
    T0 = sweep.blob(nx, ny, nz)
    torch.cuda.synchronize()
    dt = sweep.cfl_dt(nx, ny, nz, cfl=0.5)
    h = (float(nx), float(ny), float(nz))
    types, vals = BCS["hrl"]
    T64 = T0.clone()
    api.weno5_advect(ctx, T64, *V, dt, *h, types, vals, abi.WENO_V1, abi.FP64)
    T32 = T0.float().permute(2, 1, 0).contiguous().permute(2, 1, 0)
    V32 = [v.float().permute(2, 1, 0).contiguous().permute(2, 1, 0) for v in V]
    api.weno5_advect_f32(ctx, T32, *V32, dt, *h, types, vals, abi.WENO_V1)
    ctx.synchronize()
    inner = (slice(1, -1),) * 3
    ref = T64[inner]
    assert bool(torch.isfinite(T32[inner]).all())
    assert float((T32[inner].double() - ref).abs().max()) <= 1e-6 * float(ref.abs().max())


def test_sweep_f32_keeps_a_uniform_field(ctx):
    """All differences vanish: a uniform field is advected exactly (Neumann walls)."""
    for n in (19, 67):
        Vd = [v.float().permute(2, 1, 0).contiguous().permute(2, 1, 0) for v in sweep.curl_velocity(n, n, n, seed=6)]
        T = ht.zeros(n + 2, n + 2, n + 2, dtype=torch.float32) + 0.625
        api.weno5_advect_f32(ctx, T, *Vd, sweep.cfl_dt(n, n, n), float(n), float(n), float(n), [0] * 6, [0.0] * 6,
                             abi.WENO_V1)
        assert bool((T == 0.625).all()), n


def test_sweep_f32_rejects_float64(ctx):
    n = 8
    Vd = sweep.curl_velocity(n, n, n, seed=6)
    with pytest.raises(ValueError):
        api.weno5_advect_f32(ctx, sweep.blob(n, n, n), *Vd, 0.01, 8.0, 8.0, 8.0, [0] * 6, [0.0] * 6)
