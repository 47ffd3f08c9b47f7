"""Named DYREL iteration entry points and context tuning validation."""
import numpy as np
import pytest

import hydrothermal3d_gb300 as ht
from hydrothermal3d_gb300 import abi

pytestmark = pytest.mark.gpu


def _fields(n, seed):
    rng = np.random.default_rng(seed)
    nx, ny, nz = n
    X = np.asfortranarray(rng.uniform(-1, 1, (nx + 2, ny + 2, nz + 2)))
    R = np.asfortranarray(rng.uniform(-1, 1, (nx, ny, nz)))
    k = [np.asfortranarray(rng.uniform(0.5, 2, s)) for s in ((nx + 1, ny, nz), (nx, ny + 1, nz), (nx, ny, nz + 1))]
    PC = np.asfortranarray(rng.uniform(50, 100, (nx, ny, nz)))
    return X, R, k, PC


@pytest.mark.parametrize("which", ["thermal", "darcy"])
def test_named_iterations_equal_generic(ctx, which):
    n = (13, 9, 7)
    X, R, k, PC = _fields(n, 61)
    bt, bv = abi.int6(0, 0, 1, 1, 0, 0), abi.dbl6(0, 0, 1.0, 0.0, 0, 0)
    d = (1 / 13, 1 / 9, 1 / 7)
    cX = 40.0 if which == "thermal" else 0.0
    outs = []
    for named in (False, True):
        Xd, Rd, Pd, F0 = ht.from_numpy(X), ht.from_numpy(R), ht.from_numpy(PC), ht.zeros(*n)
        kd = [ht.from_numpy(a) for a in k]
        common = (Rd.data_ptr(), kd[0].data_ptr(), kd[1].data_ptr(), kd[2].data_ptr(), Pd.data_ptr(), F0.data_ptr())
        if not named:
            ctx.call("ht3d_dyrel_iterate", Xd.data_ptr(), *common, cX, *d, bt, bv, 0.9, 0.05, 0.002, 11, *n)
        elif which == "thermal":
            ctx.call("ht3d_dyrel_thermal_iterate", 11, Xd.data_ptr(), *common, cX, *d, bt, bv, 0.9, 0.05, 0.002, *n)
        else:
            ctx.call("ht3d_dyrel_darcy_iterate", 11, Xd.data_ptr(), *common, *d, bt, bv, 0.9, 0.05, 0.002, *n)
        outs.append((ht.to_numpy(Xd), ht.to_numpy(F0)))
    np.testing.assert_array_equal(outs[0][0], outs[1][0])
    np.testing.assert_array_equal(outs[0][1], outs[1][1])


@pytest.mark.parametrize("key,value", [(abi.TUNE_DYREL_VARIANT, 3), (abi.TUNE_MIXED_REFRESH, -1),
                                       (abi.TUNE_TIME_INNER, 2), (abi.TUNE_ENS_BLOCK, 100),
                                       (abi.TUNE_ENS_GRAPH, 5), (abi.TUNE_TEMPORAL, -3), (abi.TUNE_WAIT_TEST, -1),
                                       (abi.TUNE_ENS_TILE, 7), (99, 0)])
def test_tuning_rejects_bad_values(ctx, key, value):
    assert ctx.lib.ht3d_ctx_set_tuning(ctx.ptr, key, value) == abi.ERR_ARG
