"""Error paths: bad arguments, NaN residuals and divergence are reported as
status codes (the reference calls error()), never by trapping the GPU."""
import numpy as np
import pytest

import hydrothermal3d_gb300 as ht
from hydrothermal3d_gb300 import api, abi

pytestmark = pytest.mark.gpu


def _fields(n):
    rng = np.random.default_rng(41)
    nx, ny, nz = n
    X = np.asfortranarray(rng.uniform(0, 1, (nx + 2, ny + 2, nz + 2)))
    R = np.asfortranarray(rng.uniform(-1, 1, (nx, ny, nz)))
    k = [np.ones(s, order="F") for s in ((nx + 1, ny, nz), (nx, ny + 1, nz), (nx, ny, nz + 1))]
    return X, R, k


@pytest.mark.parametrize("prec", [abi.FP64, abi.MIXED])
def test_nan_input_reports_nan(ctx, prec):
    n = (8, 8, 8)
    X, R, k = _fields(n)
    R[3, 3, 3] = np.nan
    Xd = ht.from_numpy(X)
    with pytest.raises(ht.Ht3dError) as e:
        api.dyrel_solve_dimless(ctx, Xd, ht.from_numpy(R), *[ht.from_numpy(a) for a in k], 10.0, .1, .1, .1,
                                [0] * 6, [0.0] * 6, abi.DyrelParams.reference(), ht.zeros(*n), ht.zeros(*n), prec)
    assert e.value.status == abi.ERR_NAN
    # the context stays usable after the error
    a = ht.from_numpy(np.asfortranarray(np.arange(8.0).reshape(2, 2, 2)))
    assert api.sum_g(ctx, a) == 28.0


def test_divergence_reports_diverged(ctx):
    n = (8, 8, 8)
    X, R, k = _fields(n)
    prm = abi.DyrelParams.reference(nitout=5)
    prm.cfl = 3.0  # pseudo-time step far beyond the stability limit
    with pytest.raises(ht.Ht3dError) as e:
        api.dyrel_solve_dimless(ctx, ht.from_numpy(X), ht.from_numpy(R), *[ht.from_numpy(a) for a in k], 0.0, .1, .1,
                                .1, [1] * 6, [0.0] * 6, prm, ht.zeros(*n), ht.zeros(*n), abi.FP64)
    assert e.value.status == abi.ERR_DIVERGED


def test_bad_arguments(ctx):
    n = (4, 4, 4)
    X, R, k = _fields(n)
    with pytest.raises(ValueError):  # wrong staggering
        api.ComputeFlux(ctx, ht.zeros(4, 4, 4), ht.zeros(4, 5, 4), ht.zeros(4, 4, 5), *[ht.from_numpy(a) for a in k],
                        ht.from_numpy(X), 1.0, 1.0, 1.0)
    with pytest.raises(ValueError):  # row-major tensor
        import torch
        api.Multiply(ctx, torch.zeros(4, 4, 4, dtype=torch.float64, device="cuda"), ht.zeros(4, 4, 4), ht.zeros(4, 4, 4))
    with pytest.raises(ht.Ht3dError) as e:  # WENO needs n >= 3
        api.weno5_advect(ctx, ht.zeros(4, 4, 4), ht.zeros(3, 2, 2), ht.zeros(2, 3, 2), ht.zeros(2, 2, 3), 0.1, 1, 1, 1,
                         [0] * 6, [0.0] * 6)
    assert e.value.status == abi.ERR_ARG
    with pytest.raises(ht.Ht3dError) as e:  # BC type 2 is not a face BC of the diffusion solver
        api.SetFaceBCs(ctx, ht.from_numpy(X), [2] * 6, [0.0] * 6)
    assert e.value.status == abi.ERR_ARG
