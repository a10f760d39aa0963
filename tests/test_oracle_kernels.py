"""tests/test_kernels.jl restated for the oracle's Wendland kernels, plus an
exact check of the oracle's evaluation against the closed form in rationals.

Reference: tests/test_kernels.jl:20-43 (h = 0.42, TOL = 0.01, Simpson rule
with N = 1000 as at :8-17), kernels.jl:108-195 for the closed forms.
"""
import math
from fractions import Fraction

import pytest

TOL = 0.01
N = 1000


def simpson_rule(f, a, b, n=N):
    """tests/test_kernels.jl:8-17 (the same composite rule, same loop bounds)."""
    I = 0.0
    h = (b - a) / n
    for i in range(1, n):
        _a = a + i * h
        _b = a + (i + 1) * h
        I += h / 6.0 * (f(_a) + 4.0 * f(0.5 * (_a + _b)) + f(_b))
    return I


@pytest.mark.parametrize("dim", [2, 3])
def test_local_kernel(oracle_mod, dim):
    h = 0.42
    f = lambda r: oracle_mod.kernel_w(dim, h, r)
    rdf = lambda r: oracle_mod.kernel_rdw(dim, h, r)
    df = lambda r: r * rdf(r)
    assert f(4.0) == 0.0
    assert math.isfinite(f(0.0))
    if dim == 2:
        integral = simpson_rule(lambda r: 2.0 * math.pi * r * f(r), 0.0, h)
    else:
        integral = simpson_rule(lambda r: 4.0 * math.pi * r * r * f(r), 0.0, h)
    assert integral == pytest.approx(1.0, rel=TOL)
    assert df(4.0) == 0.0
    assert math.isfinite(df(0.0))
    integral = simpson_rule(df, 0.2, 0.3)
    assert integral == pytest.approx(f(0.3) - f(0.2), rel=0.01)
    assert rdf(4.0) == 0.0
    assert math.isfinite(rdf(0.0))
    assert rdf(0.1) == pytest.approx(df(0.1) / 0.1, rel=TOL)


@pytest.mark.parametrize("dim", [2, 3])
def test_kernel_closed_form(oracle_mod, dim):
    """W = C (1-x)^4 (1+4x) / h^d and rDW = -C' (1-x)^3 / h^(d+2) in exact
    rational arithmetic (kernels.jl:108-195); the oracle's rounded evaluation
    must agree to a few ulp."""
    C = {2: (Fraction(2.228169203286535), Fraction(-44.563384065730695)),
         3: (Fraction(3.3422538049298023), Fraction(-66.84507609859604))}[dim]
    h = 0.0473
    H = Fraction(h)
    # x = r * (1/h) (a reading @fastmath permits) lands within an ulp of 1 at
    # r = h, where W is ~1e-60 instead of exactly 0
    assert abs(oracle_mod.kernel_w(dim, h, h)) < 1e-40
    for r in [0.0, 0.001, 0.0123, 0.02, 0.03, 0.0471]:
        x = Fraction(r) / H
        w = C[0] * (1 - x) ** 4 * (1 + 4 * x) / H ** dim
        rdw = C[1] * (1 - x) ** 3 / H ** (dim + 2)
        # x = r*(1/h) carries a few ulp; (1-x)^4 amplifies that by 4/(1-x)
        tol = 4e-15 + 8 * 2.2e-16 / max(1.0 - r / h, 1e-3)
        assert oracle_mod.kernel_w(dim, h, r) == pytest.approx(float(w), rel=tol, abs=1e-300)
        assert oracle_mod.kernel_rdw(dim, h, r) == pytest.approx(float(rdw), rel=tol, abs=1e-300)
    assert oracle_mod.kernel_w(dim, h, h * (1 + 1e-15)) == 0.0
