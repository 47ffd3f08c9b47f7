"""The library's exponentials (hydrothermal3d_gb300/csrc/expo.h: e^x and 10^x,
used by the fluid-viscosity and permeability laws) against 40-digit decimal
arithmetic, through the CPU oracle that compiles the same header.  CUDA
documents its exp and exp10 at 1 ulp; these stay below that over the whole
finite range, including results in the subnormal range."""
import math
import os
import sys
from decimal import Decimal, getcontext

import numpy as np
import pytest

import oracle

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "hydrothermal3d_gb300", "csrc")


def _ulp(y: Decimal) -> Decimal:
    if y == 0:
        return Decimal(2) ** -1074
    e = math.frexp(float(y))[1] if float(y) != 0 else -1074
    return Decimal(2) ** max(e - 53, -1074)


def _ulp_errors(which, xs, exact):
    getcontext().prec = 40
    out = []
    for x in xs:
        got = oracle.law(which, float(x))
        ref = exact(Decimal(float(x)))
        if ref > Decimal("1.7976931348623157e308"):
            assert got == math.inf
            continue
        out.append(float(abs(Decimal(got) - ref) / _ulp(ref)))
    return np.array(out)


def test_generated_constants_match_the_header():
    sys.path.insert(0, CSRC)
    try:
        import gen_expo
    finally:
        sys.path.pop(0)
    text = open(os.path.join(CSRC, "expo.h")).read()
    body = text.split("// BEGIN generated constants\n", 1)[1].split("\n// END generated constants", 1)[0]
    assert body == gen_expo.block()


def test_exp_below_one_ulp():
    rng = np.random.default_rng(11)
    xs = np.concatenate([rng.uniform(-745.0, 709.7, 3000), rng.uniform(-1, 1, 1000), rng.uniform(-0.02, 0.02, 500),
                         [0.0, 1.0, -1.0, 1e-300, -1e-300, 709.78, 709.7827, -708.39, -720.5, -744.4, -745.1,
                          math.log(2.0), 50 * math.log(2.0)]])
    err = _ulp_errors(10, xs, lambda d: d.exp())
    assert err.max() < 1.0, err.max()
    assert oracle.law(10, 0.0) == 1.0
    assert oracle.law(10, -746.0) == 0.0 and oracle.law(10, 710.0) == math.inf
    assert math.isnan(oracle.law(10, math.nan))


def test_exp10_below_one_ulp():
    rng = np.random.default_rng(12)
    ten = Decimal(10)
    xs = np.concatenate([rng.uniform(-323.3, 308.25, 3000), rng.uniform(0.1, 1.7, 1500),
                         [0.0, 1.0, 2.0, 3.0, -1.0, 0.5, 308.25, -307.5, -310.2, -323.3, 1e-300]])
    err = _ulp_errors(11, xs, lambda d: ten ** d)
    assert err.max() < 1.0, err.max()
    assert oracle.law(11, 0.0) == 1.0
    assert oracle.law(11, -324.0) == 0.0 and oracle.law(11, 309.0) == math.inf


@pytest.mark.parametrize("T", [293.15, 400.0, 873.15, 1200.0])
def test_viscosity_law_uses_the_exponential(T):
    """mu_f(T) = 2.414e-5 * 10^(247.8/(T-140)) (Dimensional/HydroThermal3D_v18.jl:37)
    to 1 ulp of the 40-digit value."""
    getcontext().prec = 40
    x = 247.8 / (T - 140.0)
    ref = Decimal(2.414e-5) * (Decimal(10) ** Decimal(x))
    got = oracle.law(7, T)
    assert abs(Decimal(got) - ref) <= 2 * _ulp(ref)
