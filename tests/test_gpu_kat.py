"""Known-answer physics through the GPU solver and time step (cases in
kat_cases.py): the y-column geotherm against the exact 1-D solve, and the
Horton-Rogers-Lapwood onset growth factors, for the plain FP64 and the
mixed form; the reference's crustal geotherm benchmark through the
dimensional step."""
import numpy as np
import pytest

import hydrothermal3d_gb300 as ht
from hydrothermal3d_gb300 import api, abi
from kat_cases import (GEO_N, GEO_BC, geotherm_case, geotherm_exact, geotherm_params, ONSET_N, ONSET_STEPS,
                       onset_case, onset_factor, GEO18_N, geotherm_v18_case, geotherm_v18_exact, geotherm_v18_ky)

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec,tol", [(abi.FP64, 1e-12), (abi.MIXED, 1e-10)])
def test_geotherm_column_matches_1d_solve(ctx, prec, tol):
    nx, ny, nz = GEO_N
    c = geotherm_case()
    X = ht.zeros(nx + 2, ny + 2, nz + 2)
    F, F0 = ht.zeros(nx, ny, nz), ht.zeros(nx, ny, nz)
    st = api.dyrel_solve_dimless(ctx, X, ht.from_numpy(c["R"]), ht.from_numpy(c["kx"]), ht.from_numpy(c["ky"]),
                                 ht.from_numpy(c["kz"]), 0.0, *c["d"], *GEO_BC, geotherm_params(), F, F0, prec)
    assert st.status == 0
    col = ht.to_numpy(X)[1:-1, 1:-1, 1:-1]
    Tex = geotherm_exact(c)
    assert np.abs(col - Tex[None, :, None]).max() <= tol * np.abs(Tex).max()


@pytest.mark.parametrize("prec", [abi.FP64, abi.MIXED])
@pytest.mark.parametrize("Ra", [20.0, 80.0])
def test_hrl_onset_growth_factor(ctx, orc, prec, Ra):
    """The GPU step's mode amplitudes follow the oracle's (FP64: to 1e-12,
    mixed: to 1e-5 relative) and the linear growth factor."""
    n = ONSET_N
    shapes = ((n + 1, n, n), (n, n + 1, n), (n, n, n + 1))
    T, P, ktv, kfv, p, amplitude = onset_case(Ra)
    To, Po = T.copy(order="F"), P.copy(order="F")
    po = onset_case(Ra)[4]
    Vo = [np.zeros(s, order="F") for s in shapes]
    Td, Pd, ktd, kfd = (ht.from_numpy(a) for a in (T, P, ktv, kfv))
    Vd = [ht.zeros(*s) for s in shapes]
    a_gpu, a_orc = [amplitude(T[1:-1, 1:-1, 1:-1])], [amplitude(T[1:-1, 1:-1, 1:-1])]
    for _ in range(ONSET_STEPS):
        s, _, _ = orc.step_hrl(To, Po, ktv, kfv, *Vo, po)
        assert s == 0
        gt, gd = api.step_hrl(ctx, Td, Pd, ktd, kfd, *Vd, p, prec)
        assert gt.status == 0 and gd.status == 0
        a_orc.append(amplitude(To[1:-1, 1:-1, 1:-1]))
        a_gpu.append(amplitude(ht.to_numpy(Td)[1:-1, 1:-1, 1:-1]))
    a_gpu, a_orc = np.array(a_gpu), np.array(a_orc)
    tol = 1e-12 if prec == abi.FP64 else 1e-5
    assert np.abs(a_gpu - a_orc).max() <= tol * np.abs(a_orc).max()
    ratios = a_gpu[1:] / a_gpu[:-1]
    G = onset_factor(Ra)
    assert np.all(np.abs(ratios - G) <= 5e-3 * G)


def test_crustal_geotherm_benchmark_steady_state(ctx, orc):
    """Dimensional/Benchmarks/Geotherm_1D_weights.jl through ht3d_step_v18
    (it = 0, steady thermal solve): the profile marched down from the
    surface with the basal flux through every rock face, to 1e-11."""
    nx, ny, nz = GEO18_N
    c = geotherm_v18_case()
    ky = geotherm_v18_ky(orc, c)
    T, P = ht.from_numpy(c["T"]), ht.from_numpy(c["P"])
    V = [ht.zeros(nx + 1, ny, nz), ht.zeros(nx, ny + 1, nz), ht.zeros(nx, ny, nz + 1)]
    gt, _ = api.step_v18(ctx, T, P, ht.from_numpy(c["phc"]), ht.from_numpy(c["phv"]), ht.from_numpy(c["wN"]), None,
                         *V, c["params"])
    assert gt.status == 0 and gt.converged
    exact = geotherm_v18_exact(c, ky)
    got = ht.to_numpy(T)[1:-1, 1:c["js"] + 2, 1:-1]
    assert np.abs(got - exact).max() <= 1e-11 * np.abs(exact).max()

