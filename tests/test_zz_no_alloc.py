"""The allocation-free DYREL iteration (ht3d_dyrel_iterate_noalloc).

It serves callers that cannot let the library allocate device memory; it
must give the same bits as ht3d_dyrel_iterate (inner cells, face ghosts and
F0), twice in a row, allocate nothing after its first call on a device, and
refuse grids larger than its fixed scratch.  Collected last so a failure here
comes after every other test.
"""
import numpy as np
import pytest
import torch

import hydrothermal3d_gb300 as ht
from hydrothermal3d_gb300 import abi

pytestmark = pytest.mark.gpu


def _fields(n, seed=5):
    nx, ny, nz = n
    rng = np.random.default_rng(seed)
    X = ht.from_numpy(rng.uniform(0, 1, (nx + 2, ny + 2, nz + 2)))
    R = ht.from_numpy(rng.uniform(-1, 1, (nx, ny, nz)))
    k = [ht.from_numpy(rng.uniform(0.5, 2, s)) for s in ((nx + 1, ny, nz), (nx, ny + 1, nz), (nx, ny, nz + 1))]
    PC = ht.from_numpy(rng.uniform(3, 6, (nx, ny, nz)) * nx * nx)
    F0 = ht.zeros(nx, ny, nz)
    return X, R, k, PC, F0


def _args(X, R, k, PC, F0, n, n_iter):
    nx, ny, nz = n
    return (X.data_ptr(), R.data_ptr(), k[0].data_ptr(), k[1].data_ptr(), k[2].data_ptr(), PC.data_ptr(),
            F0.data_ptr(), 20.0, 1.0 / nx, 1.0 / ny, 1.0 / nz, abi.int6(0, 0, 1, 1, 0, 1),
            abi.dbl6(0, 0, 1.0, 0.0, 0, 0.5), 0.97, 0.02, 0.015, n_iter, nx, ny, nz)


def _inner_and_faces(shape):
    """Cells with at most one index on the ghost shell: inner cells and face
    ghosts (edge and corner ghosts are not written by either path)."""
    on = [np.zeros(s, bool) for s in shape]
    for o in on:
        o[[0, -1]] = True
    count = on[0][:, None, None].astype(int) + on[1][None, :, None] + on[2][None, None, :]
    return count <= 1


@pytest.mark.parametrize("n,n_iter", [((40, 30, 20), 17), ((7, 5, 3), 17), ((40, 30, 20), 16), ((9, 11, 13), 1)])
def test_noalloc_matches_dyrel_iterate_twice(ctx, n, n_iter):
    """Odd counts end in the scratch array and copy back; even counts end in X."""
    lib = ctx.lib
    X, R, k, PC, F0 = _fields(n)
    Xa, F0a = X.clone(), F0.clone()
    stream = torch.cuda.current_stream().cuda_stream
    m = _inner_and_faces(X.shape)
    for call in range(2):  # two calls in a row, each continuing from the last state
        ctx.call("ht3d_dyrel_iterate", *_args(X, R, k, PC, F0, n, n_iter))
        st = lib.ht3d_dyrel_iterate_noalloc(*_args(Xa, R, k, PC, F0a, n, n_iter), stream)
        torch.cuda.synchronize()
        assert st == abi.OK
        a, b = ht.to_numpy(Xa), ht.to_numpy(X)
        np.testing.assert_array_equal(a[m], b[m])
        np.testing.assert_array_equal(ht.to_numpy(F0a), ht.to_numpy(F0))


def test_noalloc_allocates_nothing_after_first_call(ctx):
    n = (24, 24, 24)
    X, R, k, PC, F0 = _fields(n, seed=6)
    lib = ctx.lib
    stream = torch.cuda.current_stream().cuda_stream
    assert lib.ht3d_dyrel_iterate_noalloc(*_args(X, R, k, PC, F0, n, 3), stream) == abi.OK  # set-up call
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        assert lib.ht3d_dyrel_iterate_noalloc(*_args(X, R, k, PC, F0, n, 5), stream) == abi.OK
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0


def test_noalloc_rejects_grids_beyond_its_scratch(ctx):
    # (nx+2)(ny+2)(nz+2) = 102^3 > 2^20: refused before anything is launched
    X, R, k, PC, F0 = _fields((4, 4, 4), seed=7)
    st = ctx.lib.ht3d_dyrel_iterate_noalloc(*_args(X, R, k, PC, F0, (100, 100, 100), 1), None)
    assert st == abi.ERR_SCRATCH
    assert b"static scratch" in ctx.lib.ht3d_status_string(st)
